// Tile reduction of the K values: the element contributions of a resident
// pattern summed without the per-contribution index lists of reduce_win_k.
//
// The columns of the CSC pattern are cut into tiles (consecutive columns, at
// most kTileMaxNz nonzeros and kTileMaxContrib contributions each).  For each
// tile a program is built once per pattern:
//   - the distinct elements contributing to the tile, as offsets from the
//     tile's smallest element;
//   - the tile's nonzeros in order of their contributor count (a stable
//     counting sort), so that the lanes of a warp issue about as many FP64
//     adds as their nonzeros need;
//   - per nonzero its first code (its position in the tile << 16 | the index
//     of its first contribution in the tile's value table), and its further
//     codes, stored count class by count class, contribution-major, so that
//     each round of a warp reads consecutive codes.
// A value table holds V values per element of the tile: the element's K
// record (V = S), or for the exact-rational T6 heat record the 14 values its
// 8 bases expand to (t6r_table), entry-major (value j of the tile's element
// k at j * nel + k, so that the threads staging consecutive elements write
// consecutive words).  Every nonzero adds its contributions in
// slot order -- the order of the contributor lists of the pattern, which is
// the order in which SparseArrays.sparse adds duplicates -- so the values are
// the bits of reduce_values.
//
// A program is one contiguous, 16-byte aligned blob (count classes, element
// offsets, first codes, further codes), copied into shared memory with
// vector loads (once per tile, or once per run of consecutive tiles of one
// program in tile_run_k).  Tiles whose programs are equal word for word (the
// tiles of a structured mesh away from its boundary are translates of a few)
// share one copy: only distinct programs are kept, and per step a tile reads
// its own first nonzero and smallest element and the blob of its program,
// which stays in L2.
#include <algorithm>
#include <unordered_map>
#include <vector>

#include "sysmat.cuh"
#include "t6r.cuh"

namespace elfel {

namespace {

constexpr int kTT = kTileThreads;

struct TileBuildArgs {
  const int64_t* colptr;
  const int32_t* cptr;
  const int32_t* contrib;
  int S, V;
  FastDiv sdiv;
  uint8_t map[kTileMaxS];
  int emax;
};

// Byte layout of a tile program: count classes (kTileMaxClass + 2 uint16,
// padded to 48 bytes), element offsets (int32), first codes (uint32), further
// codes (uint16), each part padded to 16 bytes.
struct BlobLayout {
  int el, f, r, bytes;
};
__host__ __device__ __forceinline__ int pad16(int b) { return (b + 15) & ~15; }
__host__ __device__ __forceinline__ BlobLayout blob_layout(int nel, int nz, int nc) {
  BlobLayout L;
  L.el = 48;
  L.f = L.el + pad16(4 * nel);
  L.r = L.f + pad16(4 * nz);
  L.bytes = L.r + pad16(2 * (nc - nz));
  return L;
}

// cq[k] = cptr[colptr[k]]: the first contribution of each column (k <= ncol).
__global__ void cptr_at_cols_k(const int64_t* __restrict__ colptr, const int32_t* __restrict__ cptr, int64_t ncol,
                               int32_t* __restrict__ cq) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k <= ncol; k += (int64_t)gridDim.x * blockDim.x)
    cq[k] = cptr[colptr[k]];
}

// Sort n <= kTileMaxContrib ints in shared memory ascending (bitonic network
// over the next power of two, padded with INT32_MAX).
__device__ void smem_sort(int32_t* a, int n) {
  int np = 1;
  while (np < n) np <<= 1;
  for (int i = n + threadIdx.x; i < np; i += blockDim.x) a[i] = 0x7fffffff;
  __syncthreads();
  for (int size = 2; size <= np; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < np / 2; i += blockDim.x) {
        const int lo = 2 * i - (i & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const int32_t x = a[lo], y = a[hi];
        if ((x > y) == up) {
          a[lo] = y;
          a[hi] = x;
        }
      }
      __syncthreads();
    }
  }
}

// First pass: the size of each tile (nonzeros, contributions, distinct
// elements, largest contributor count); tiles beyond the limits are marked.
__global__ void __launch_bounds__(kTT) tile_count_k(TileHdr* __restrict__ hdr, int64_t ntiles, TileBuildArgs a) {
  __shared__ int32_t el[kTileMaxContrib];
  __shared__ int red[2];
  const int64_t t = blockIdx.x;
  if (t >= ntiles) return;
  TileHdr H = hdr[t];
  const int64_t p0 = a.colptr[H.col0], p1 = a.colptr[H.col0 + H.ncols];
  const int64_t q0 = a.cptr[p0], q1 = a.cptr[p1];
  H.p0 = p0;
  H.q0 = q0;
  H.nz = (int32_t)(p1 - p0);
  H.nc = (int32_t)(q1 - q0);
  if (H.nz > kTileMaxNz || H.nc > kTileMaxContrib || H.nz == 0) {
    if (threadIdx.x == 0) {
      H.flags = H.nz == 0 ? kTileEmpty : kTileFallback;
      H.nel = 0;
      H.maxcnt = 0;
      hdr[t] = H;
    }
    return;
  }
  if (threadIdx.x == 0) red[0] = red[1] = 0;
  for (int i = threadIdx.x; i < H.nc; i += kTT) el[i] = (int32_t)a.sdiv.div((uint32_t)a.contrib[q0 + i]);
  int mx = 0;
  for (int i = threadIdx.x; i < H.nz; i += kTT) mx = max(mx, a.cptr[p0 + i + 1] - a.cptr[p0 + i]);
  smem_sort(el, H.nc);  // contains __syncthreads
  int nuniq = 0;
  for (int i = threadIdx.x; i < H.nc; i += kTT) nuniq += (i == 0 || el[i] != el[i - 1]) ? 1 : 0;
  atomicAdd(&red[0], nuniq);
  atomicMax(&red[1], mx);
  __syncthreads();
  if (threadIdx.x == 0) {
    H.nel = red[0];
    H.maxcnt = red[1];
    H.emin = el[0];
    H.flags = (red[0] > a.emax || red[1] > kTileMaxClass) ? kTileSplit : 0;
    hdr[t] = H;
  }
}

// Second pass: the program of every tile within the limits, written at the
// tile's blob offset.
__global__ void __launch_bounds__(kTT) tile_build_k(TileHdr* __restrict__ hdr, int64_t ntiles, TileBuildArgs a,
                                                    uint8_t* __restrict__ blob) {
  __shared__ int32_t el[kTileMaxContrib];
  __shared__ uint8_t cnt[kTileMaxNz];
  __shared__ uint16_t sidx[kTileMaxNz];
  __shared__ int cstart[kTileMaxClass + 2], rbase[kTileMaxClass + 2];
  __shared__ int nuniq;
  __shared__ int wsum[kTT / 32];
  const int64_t t = blockIdx.x;
  if (t >= ntiles) return;
  const TileHdr H = hdr[t];
  if (H.flags) return;
  const int64_t p0 = H.p0, q0 = H.q0;
  const int nz = H.nz, nc = H.nc;
  const BlobLayout L = blob_layout(H.nel, nz, nc);
  uint8_t* b0 = blob + H.boff;
  uint16_t* cls = reinterpret_cast<uint16_t*>(b0);
  int32_t* elist = reinterpret_cast<int32_t*>(b0 + L.el);
  uint32_t* firsts = reinterpret_cast<uint32_t*>(b0 + L.f);
  uint16_t* rest = reinterpret_cast<uint16_t*>(b0 + L.r);
  for (int k = threadIdx.x; k < L.bytes / 4; k += kTT) reinterpret_cast<uint32_t*>(b0)[k] = 0u;  // the padding
  for (int i = threadIdx.x; i < nc; i += kTT) el[i] = (int32_t)a.sdiv.div((uint32_t)a.contrib[q0 + i]);
  for (int i = threadIdx.x; i < nz; i += kTT) cnt[i] = (uint8_t)(a.cptr[p0 + i + 1] - a.cptr[p0 + i]);
  if (threadIdx.x < kTileMaxClass + 2) cstart[threadIdx.x] = 0;
  smem_sort(el, nc);  // contains __syncthreads (after the padding writes)
  // distinct elements, compacted in place by one warp (ordered ballots)
  if (threadIdx.x < 32) {
    int w = 0;
    for (int base = 0; base < nc; base += 32) {
      const int i = base + threadIdx.x;
      const bool keep = i < nc && (i == 0 || el[i] != el[i - 1]);
      const int32_t v = i < nc ? el[i] : 0;
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      __syncwarp();
      if (keep) el[w + __popc(m & ((1u << threadIdx.x) - 1))] = v;
      w += __popc(m);
      __syncwarp();
    }
    if (threadIdx.x == 0) nuniq = w;
  }
  __syncthreads();
  const int nel = nuniq;
  const int32_t emin = el[0];
  for (int k = threadIdx.x; k < nel; k += kTT) elist[k] = el[k] - emin;
  // count classes and the stable order within each class
  for (int i = threadIdx.x; i < nz; i += kTT) atomicAdd(&cstart[cnt[i] + 1], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0, rb = 0;
    for (int c = 1; c <= kTileMaxClass + 1; ++c) {
      const int n = c <= kTileMaxClass ? cstart[c + 1] : 0;
      cstart[c] = run;
      rbase[c] = rb;
      run += n;
      rb += n * (c - 1);
    }
    cstart[0] = 0;
  }
  __syncthreads();
  for (int c = 1; c <= kTileMaxClass; ++c) {
    int before = cstart[c];
    for (int base = 0; base < nz; base += kTT) {
      const int i = base + threadIdx.x;
      const bool in = i < nz && cnt[i] == c;
      const unsigned m = __ballot_sync(0xffffffffu, in);
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      if (lane == 0) wsum[wid] = __popc(m);
      __syncthreads();
      int off = before;
      for (int w = 0; w < wid; ++w) off += wsum[w];
      if (in) sidx[i] = (uint16_t)(off + __popc(m & ((1u << lane) - 1)));
      int tot = 0;
      for (int w = 0; w < kTT / 32; ++w) tot += wsum[w];
      __syncthreads();
      before += tot;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kTileMaxClass + 2; k += kTT)
    cls[k] = (uint16_t)(k == kTileMaxClass + 1 ? nz : cstart[k]);
  // codes: table index of every contribution
  for (int i = threadIdx.x; i < nz; i += kTT) {
    const int c = cnt[i];
    const int si = sidx[i];
    const int nclass = cstart[c + 1] - cstart[c];
    const int32_t b = a.cptr[p0 + i];
    for (int k = 0; k < c; ++k) {
      const uint32_t st = (uint32_t)a.contrib[b + k];
      const uint32_t e = a.sdiv.div(st);
      const int s = (int)(st - e * (uint32_t)a.S);
      int lo = 0, hi = nel - 1;  // e's index in the distinct list
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (el[mid] < (int32_t)e) lo = mid + 1; else hi = mid;
      }
      const uint32_t code = (uint32_t)(a.map[s] * nel + lo);  // entry-major value table
      if (k == 0)
        firsts[si] = ((uint32_t)i << 16) | code;
      else
        rest[rbase[c] + (k - 1) * nclass + (si - cstart[c])] = (uint16_t)code;
    }
  }
  if (threadIdx.x == 0) {
    TileHdr h = H;
    h.emin = emin;
    h.nel = nel;
    hdr[t] = h;
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// A 64-bit digest of each program: a sum of mixed (word, index) pairs, so
// that it does not depend on the order threads add them.
__global__ void __launch_bounds__(kTT) tile_hash_k(const TileHdr* __restrict__ hdr, int64_t ntiles,
                                                   const uint8_t* __restrict__ blob, uint64_t* __restrict__ hash) {
  __shared__ unsigned long long part;
  const int64_t t = blockIdx.x;
  if (t >= ntiles) return;
  const TileHdr H = hdr[t];
  if (H.flags) {
    if (threadIdx.x == 0) hash[t] = 0;
    return;
  }
  if (threadIdx.x == 0) part = 0;
  __syncthreads();
  const BlobLayout L = blob_layout(H.nel, H.nz, H.nc);
  const uint32_t* w = reinterpret_cast<const uint32_t*>(blob + H.boff);
  uint64_t h = 0;
  for (int k = threadIdx.x; k < L.bytes / 4; k += kTT) h += mix64(((uint64_t)k << 32) + w[k]);
  atomicAdd(&part, (unsigned long long)h);
  __syncthreads();
  if (threadIdx.x == 0) hash[t] = mix64(part ^ ((uint64_t)H.nz << 40) ^ ((uint64_t)H.nc << 20) ^ (uint64_t)H.nel);
}

// A tile keeps its representative's program only if the two are equal word
// for word; otherwise it is its own representative.
__global__ void __launch_bounds__(kTT) tile_verify_k(TileHdr* __restrict__ hdr, int64_t ntiles,
                                                     const uint8_t* __restrict__ blob) {
  __shared__ int diff;
  const int64_t t = blockIdx.x;
  if (t >= ntiles) return;
  const TileHdr H = hdr[t];
  if (H.flags || H.prog == t) return;
  const TileHdr R = hdr[H.prog];
  if (threadIdx.x == 0) diff = (R.nz != H.nz || R.nc != H.nc || R.nel != H.nel || R.flags) ? 1 : 0;
  __syncthreads();
  if (!diff) {
    const BlobLayout L = blob_layout(H.nel, H.nz, H.nc);
    const uint32_t* a = reinterpret_cast<const uint32_t*>(blob + H.boff);
    const uint32_t* b = reinterpret_cast<const uint32_t*>(blob + R.boff);
    int d = 0;
    for (int k = threadIdx.x; k < L.bytes / 4; k += kTT) d |= a[k] != b[k];
    if (d) atomicOr(&diff, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && diff) hdr[t].prog = t;
}

// Copy of the distinct programs into the compact blob array: job j moves
// bytes[j] bytes from offset src[j] to offset dst[j] (multiples of 16).
__global__ void blob_copy_k(const int64_t* __restrict__ src, const int64_t* __restrict__ dst,
                            const int32_t* __restrict__ bytes, const uint8_t* __restrict__ from,
                            uint8_t* __restrict__ to) {
  const int j = blockIdx.x;
  const uint4* a = reinterpret_cast<const uint4*>(from + src[j]);
  uint4* b = reinterpret_cast<uint4*>(to + dst[j]);
  for (int k = threadIdx.x; k < bytes[j] / 16; k += blockDim.x) b[k] = a[k];
}

// Per-element value tables.  Full records: the S stored values.
struct RecFull {
  const double* store;
  int S;
  __device__ __forceinline__ void stage(int64_t e, double* v, int ld) const {
    for (int k = 0; k < S; ++k) v[k * ld] = __ldg(store + e * S + k);
  }
  __device__ __forceinline__ double value(uint32_t st) const { return __ldg(store + st); }
};

// The 8 bases of the exact-rational T6 record (64 bytes per element).
struct RecT6R {
  const double* bases;
  __device__ __forceinline__ void load(int64_t e, double2 (&x)[4]) const {
    const double2* p = reinterpret_cast<const double2*>(bases + e * 8);
#pragma unroll
    for (int k = 0; k < 4; ++k) x[k] = __ldg(p + k);
  }
  __device__ __forceinline__ static void expand(const double2 (&x)[4], double* v, int ld) {
    double b[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      b[2 * k] = x[k].x;
      b[2 * k + 1] = x[k].y;
    }
    t6r_table(b, v, ld);
  }
  __device__ __forceinline__ void stage(int64_t e, double* v, int ld) const {
    double2 x[4];
    load(e, x);
    expand(x, v, ld);
  }
  // stored entry st = e * 21 + s of the record
  __device__ __forceinline__ double value(uint32_t st) const {
    const uint32_t e = st / 21u, s = st - e * 21u;
    double b[8], v[kT6RTable];
#pragma unroll
    for (int k = 0; k < 8; ++k) b[k] = __ldg(bases + (int64_t)e * 8 + k);
    t6r_table(b, v);
    return v[t6r_entry((int)s)];
  }
};

constexpr int kRT = 64;                  // threads of tile_reduce_k
constexpr int kTileRun = 6;              // tiles per run of tile_run_k

// Adds of one tile: one thread per nonzero in count order (the program's
// first codes), each summing its contributions in slot order from the value
// table, the sums placed in CSC order in out.
template <int RT>
__device__ __forceinline__ void tile_adds(const uint8_t* sb, const BlobLayout& L, int nz, const double* tbl,
                                          double* out) {
  const uint16_t* cstart = reinterpret_cast<const uint16_t*>(sb);
  const uint32_t* sf = reinterpret_cast<const uint32_t*>(sb + L.f);
  const uint16_t* sr = reinterpret_cast<const uint16_t*>(sb + L.r);
  int c = 1, rb = 0;  // class of the current nonzero and the start of its class's further codes
#pragma unroll
  for (int j = 0; j < kTileMaxNz / RT; ++j) {
    const int i = threadIdx.x + j * RT;
    if (i < nz) {
      while (i >= cstart[c + 1]) {
        rb += (cstart[c + 1] - cstart[c]) * (c - 1);
        ++c;
      }
      const uint32_t f = sf[i];
      const int n = cstart[c + 1] - cstart[c];
      const uint16_t* r = sr + rb + (i - cstart[c]);
      double s = tbl[f & 0xffffu];
#pragma unroll 1
      for (int k = 1; k < c; ++k) s = __dadd_rn(s, tbl[r[(k - 1) * n]]);
      out[f >> 16] = s;
    }
  }
}

// One CTA per tile: the tile's program copied into shared memory while the
// value table of its elements is staged beside it, one thread per nonzero in
// count order, the tile's values written out in CSC order.
template <class Rec>
__global__ void __launch_bounds__(kRT) tile_reduce_k(const TileHdr* __restrict__ hdr, int maxnel, int V, int maxblob,
                                                     const uint8_t* __restrict__ blob,
                                                     const int32_t* __restrict__ cptr,
                                                     const int32_t* __restrict__ contrib, Rec rec,
                                                     double* __restrict__ vals) {
  extern __shared__ uint4 smq[];  // program (maxblob bytes) | value table | values
  const TileHdr H = hdr[blockIdx.x];
  if (H.flags) {
    if (H.flags & kTileEmpty) return;
    // beyond the limits: every nonzero from its contributor list
    for (int i = threadIdx.x; i < H.nz; i += kRT) {
      const int32_t b = cptr[H.p0 + i], e = cptr[H.p0 + i + 1];
      double s = rec.value((uint32_t)contrib[b]);
      for (int32_t k = b + 1; k < e; ++k) s = __dadd_rn(s, rec.value((uint32_t)contrib[k]));
      vals[H.p0 + i] = s;
    }
    return;
  }
  const BlobLayout L = blob_layout(H.nel, H.nz, H.nc);
  // the program into shared memory and, at the same time, the value table of
  // the tile's elements (their offsets read from the program in L2)
  const uint4* src = reinterpret_cast<const uint4*>(blob + H.boff);
  for (int k = threadIdx.x; k < L.bytes / 16; k += kRT) smq[k] = __ldg(src + k);
  const uint8_t* sb = reinterpret_cast<const uint8_t*>(smq);
  double* tbl = reinterpret_cast<double*>(reinterpret_cast<uint8_t*>(smq) + maxblob);
  double* out = tbl + (size_t)maxnel * V;
  const int32_t* gel = reinterpret_cast<const int32_t*>(blob + H.boff + L.el);
  for (int k = threadIdx.x; k < H.nel; k += kRT) rec.stage((int64_t)H.emin + __ldg(gel + k), tbl + k, H.nel);
  __syncthreads();
  tile_adds<kRT>(sb, L, H.nz, tbl, out);
  __syncthreads();
  for (int i = threadIdx.x; i < H.nz; i += kRT) vals[H.p0 + i] = out[i];
}

// One CTA of kRunThreads per run of consecutive tiles that read the same
// program (T6 bases).  The program is copied into shared memory once per run;
// a thread's element (its position in the program's element list, at most
// one per thread) is the same in every tile of the run, so the 8 bases of the
// next tile's element are loaded into registers before the current tile's
// adds and expanded into the value table after them: the gather of tile t + 1
// overlaps the adds of tile t.
constexpr int kRunThreads = 128;

__global__ void __launch_bounds__(kRunThreads) tile_run_k(const TileHdr* __restrict__ hdr,
                                                          const int2* __restrict__ runs, int maxnel, int maxblob,
                                                          const uint8_t* __restrict__ blob,
                                                          const int32_t* __restrict__ cptr,
                                                          const int32_t* __restrict__ contrib, RecT6R rec,
                                                          double* __restrict__ vals) {
  constexpr int RT = kRunThreads;
  extern __shared__ uint4 smq[];  // program (maxblob bytes) | value table | values
  const int2 run = runs[blockIdx.x];
  const TileHdr H0 = hdr[run.x];
  if (H0.flags) {
    // tiles beyond the limits: every nonzero from its contributor list
    for (int t = run.x; t < run.x + run.y; ++t) {
      const TileHdr H = hdr[t];
      if (H.flags & kTileEmpty) continue;
      for (int i = threadIdx.x; i < H.nz; i += RT) {
        const int32_t b = cptr[H.p0 + i], e = cptr[H.p0 + i + 1];
        double s = rec.value((uint32_t)contrib[b]);
        for (int32_t k = b + 1; k < e; ++k) s = __dadd_rn(s, rec.value((uint32_t)contrib[k]));
        vals[H.p0 + i] = s;
      }
    }
    return;
  }
  const BlobLayout L = blob_layout(H0.nel, H0.nz, H0.nc);
  const int nel = H0.nel, nz = H0.nz;
  const bool mine = (int)threadIdx.x < nel;  // the thread stages element threadIdx.x of each tile
  const int32_t eo = mine ? __ldg(reinterpret_cast<const int32_t*>(blob + H0.boff + L.el) + threadIdx.x) : 0;
  double2 x[4];
  if (mine) rec.load((int64_t)H0.emin + eo, x);
  const uint4* src = reinterpret_cast<const uint4*>(blob + H0.boff);
  for (int k = threadIdx.x; k < L.bytes / 16; k += RT) smq[k] = __ldg(src + k);
  const uint8_t* sb = reinterpret_cast<const uint8_t*>(smq);
  double* tbl = reinterpret_cast<double*>(reinterpret_cast<uint8_t*>(smq) + maxblob);
  double* out = tbl + (size_t)maxnel * kT6RTable;
  int64_t p0 = H0.p0;
  for (int t = 0; t < run.y; ++t) {
    if (mine) RecT6R::expand(x, tbl + threadIdx.x, nel);
    int64_t pn = 0;
    if (t + 1 < run.y) {
      const TileHdr* hn = hdr + run.x + t + 1;
      pn = hn->p0;
      if (mine) rec.load((int64_t)hn->emin + eo, x);
    }
    __syncthreads();  // the program and the table are in place; out is free
    tile_adds<RT>(sb, L, nz, tbl, out);
    __syncthreads();  // out is complete; the table is free
    for (int i = threadIdx.x; i < nz; i += RT) vals[p0 + i] = out[i];
    p0 = pn;
  }
}

}  // namespace

void TilePlan::release(Ctx* c) {
  runs.release(c);
  nruns = 0;
  runlen = 0;
  hdr.release(c);
  blob.release(c);
  ntiles = 0;
  built = 0;
  S = V = emax = maxblob = maxnel = 0;
  nprograms = nfallback = 0;
}

int build_tile_plan(Ctx* c, Pattern& P, int S, int V, const uint8_t* map) {
  TilePlan& T = P.tiles;
  T.release(c);
  if (P.nnz == 0 || P.ncol == 0) return ELFEL_OK;
  if (S < 1 || S > kTileMaxS || V < 1) return fail(c, ELFEL_ERR_ARG, "tile plan: record of %d entries", S);
  T.S = S;
  T.V = V;
  T.emax = std::min(kTileMaxEl, (int)(kTileTableBytes / (V * (int)sizeof(double))));
  if (T.emax * V > 0xffff) T.emax = 0xffff / V;
  // column sizes on the host: nonzeros from colptr, contributions from cptr at the column starts
  const int64_t ncol = P.ncol;
  std::vector<int64_t> colptr((size_t)ncol + 1);
  ELFEL_CUDA(c, cudaMemcpyAsync(colptr.data(), P.colptr.p, sizeof(int64_t) * (ncol + 1), cudaMemcpyDeviceToHost,
                                c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  std::vector<int32_t> cq((size_t)ncol + 1);
  {
    DBuf<int32_t> d;
    ELFEL_TRY(d.alloc(c, (size_t)ncol + 1));
    cptr_at_cols_k<<<grid_for(ncol + 1, 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(P.colptr.p, P.cptr.p,
                                                                                             ncol, d.p);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_CUDA(c, cudaMemcpyAsync(cq.data(), d.p, sizeof(int32_t) * (ncol + 1), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    d.release(c);
  }
  // greedy tiles of consecutive columns within the limits; a tile cut short
  // by a limit keeps a multiple of 4 columns, so that on a structured mesh
  // (DOFs of a grid line alternate between 2 or 4 kinds) the next tile starts
  // at the same phase and translated tiles get equal programs
  std::vector<TileHdr> tiles;
  for (int64_t c0 = 0; c0 < ncol;) {
    int64_t c1 = c0 + 1;
    while (c1 < ncol && c1 - c0 < kTileMaxCols && colptr[c1 + 1] - colptr[c0] <= kTileMaxNz &&
           (int64_t)cq[c1 + 1] - cq[c0] <= kTileMaxContrib)
      ++c1;
    if (c1 < ncol && c1 - c0 >= 8) c1 = c0 + ((c1 - c0) & ~(int64_t)3);
    TileHdr h{};
    h.col0 = (int32_t)c0;
    h.ncols = (int32_t)(c1 - c0);
    tiles.push_back(h);
    c0 = c1;
  }
  TileBuildArgs a;
  a.colptr = P.colptr.p;
  a.cptr = P.cptr.p;
  a.contrib = P.contrib.p;
  a.S = S;
  a.V = V;
  a.sdiv.init((uint32_t)S);
  memset(a.map, 0, sizeof(a.map));
  for (int s = 0; s < S; ++s) a.map[s] = map ? map[s] : (uint8_t)s;
  a.emax = T.emax;
  // count, split the tiles beyond the element or class limits, count again
  for (int round = 0;; ++round) {
    const int64_t nt = (int64_t)tiles.size();
    ELFEL_TRY(T.hdr.alloc(c, (size_t)nt));
    ELFEL_CUDA(c, cudaMemcpyAsync(T.hdr.p, tiles.data(), sizeof(TileHdr) * nt, cudaMemcpyHostToDevice, c->stream));
    tile_count_k<<<(unsigned)nt, kTT, 0, c->stream>>>(T.hdr.p, nt, a);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_CUDA(c, cudaMemcpyAsync(tiles.data(), T.hdr.p, sizeof(TileHdr) * nt, cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<TileHdr> next;
    bool split = false;
    for (const TileHdr& h : tiles) {
      if ((h.flags & kTileSplit) && h.ncols > 1 && round < 12) {
        TileHdr x{}, y{};
        x.col0 = h.col0;
        x.ncols = h.ncols / 2;
        y.col0 = h.col0 + x.ncols;
        y.ncols = h.ncols - x.ncols;
        next.push_back(x);
        next.push_back(y);
        split = true;
      } else {
        TileHdr k = h;
        if (k.flags & kTileSplit) k.flags = kTileFallback;
        next.push_back(k);
      }
    }
    tiles.swap(next);
    if (!split) break;
    T.hdr.release(c);
  }
  const int64_t nt = (int64_t)tiles.size();
  // blob offsets of the programs (tiles within the limits)
  int64_t total = 0;
  for (TileHdr& h : tiles) {
    h.boff = total;
    if (!h.flags) total += blob_layout(h.nel, h.nz, h.nc).bytes;
  }
  ELFEL_CUDA(c, cudaMemcpyAsync(T.hdr.p, tiles.data(), sizeof(TileHdr) * nt, cudaMemcpyHostToDevice, c->stream));
  T.ntiles = nt;
  DBuf<uint8_t> full;
  ELFEL_TRY(full.alloc(c, (size_t)std::max<int64_t>(16, total)));
  tile_build_k<<<(unsigned)nt, kTT, 0, c->stream>>>(T.hdr.p, nt, a, full.p);
  ELFEL_LAUNCH_CHECK(c);
  // deduplicate equal programs: digests on the device, groups on the host,
  // then a word-for-word check of every tile against its representative
  DBuf<uint64_t> hash;
  ELFEL_TRY(hash.alloc(c, (size_t)nt));
  tile_hash_k<<<(unsigned)nt, kTT, 0, c->stream>>>(T.hdr.p, nt, full.p, hash.p);
  ELFEL_LAUNCH_CHECK(c);
  std::vector<uint64_t> hh((size_t)nt);
  ELFEL_CUDA(c, cudaMemcpyAsync(hh.data(), hash.p, sizeof(uint64_t) * nt, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(tiles.data(), T.hdr.p, sizeof(TileHdr) * nt, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  hash.release(c);
  std::unordered_map<uint64_t, int32_t> first;
  first.reserve((size_t)nt);
  int64_t nfb = 0;
  for (int64_t t = 0; t < nt; ++t) {
    TileHdr& h = tiles[t];
    h.prog = (int32_t)t;
    if (h.flags) {
      nfb += (h.flags & kTileFallback) ? 1 : 0;
      continue;
    }
    auto it = first.find(hh[t]);
    if (it == first.end())
      first.emplace(hh[t], (int32_t)t);
    else
      h.prog = it->second;
  }
  ELFEL_CUDA(c, cudaMemcpyAsync(T.hdr.p, tiles.data(), sizeof(TileHdr) * nt, cudaMemcpyHostToDevice, c->stream));
  tile_verify_k<<<(unsigned)nt, kTT, 0, c->stream>>>(T.hdr.p, nt, full.p);
  ELFEL_LAUNCH_CHECK(c);
  ELFEL_CUDA(c, cudaMemcpyAsync(tiles.data(), T.hdr.p, sizeof(TileHdr) * nt, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  // keep the distinct programs only, each tile pointing at its program's copy
  std::vector<int64_t> src, dst;
  std::vector<int32_t> bytes;
  std::vector<int64_t> newoff((size_t)nt, -1);
  int64_t compact = 0;
  int maxblob = 16, maxnel = 1;
  for (int64_t t = 0; t < nt; ++t) {
    const TileHdr& h = tiles[t];
    if (h.flags || h.prog != t) continue;
    const int b = blob_layout(h.nel, h.nz, h.nc).bytes;
    src.push_back(h.boff);
    dst.push_back(compact);
    bytes.push_back(b);
    newoff[t] = compact;
    compact += b;
    maxblob = std::max(maxblob, b);
    maxnel = std::max(maxnel, h.nel);
  }
  for (int64_t t = 0; t < nt; ++t) {
    TileHdr& h = tiles[t];
    if (!h.flags) h.boff = newoff[h.prog];
  }
  const int64_t nprog = (int64_t)src.size();
  ELFEL_TRY(T.blob.alloc(c, (size_t)std::max<int64_t>(16, compact)));
  if (nprog) {
    DBuf<int64_t> ds, dd;
    DBuf<int32_t> db;
    ELFEL_TRY(ds.alloc(c, (size_t)nprog));
    ELFEL_TRY(dd.alloc(c, (size_t)nprog));
    ELFEL_TRY(db.alloc(c, (size_t)nprog));
    ELFEL_CUDA(c, cudaMemcpyAsync(ds.p, src.data(), sizeof(int64_t) * nprog, cudaMemcpyHostToDevice, c->stream));
    ELFEL_CUDA(c, cudaMemcpyAsync(dd.p, dst.data(), sizeof(int64_t) * nprog, cudaMemcpyHostToDevice, c->stream));
    ELFEL_CUDA(c, cudaMemcpyAsync(db.p, bytes.data(), sizeof(int32_t) * nprog, cudaMemcpyHostToDevice, c->stream));
    blob_copy_k<<<(unsigned)nprog, 256, 0, c->stream>>>(ds.p, dd.p, db.p, full.p, T.blob.p);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_CUDA(c, cudaMemcpyAsync(T.hdr.p, tiles.data(), sizeof(TileHdr) * nt, cudaMemcpyHostToDevice, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    ds.release(c);
    dd.release(c);
    db.release(c);
  }
  full.release(c);
  // runs of consecutive tiles of one program (translated tiles of a
  // structured mesh follow one another), or of consecutive tiles beyond the
  // limits, at most kTileRun tiles each (ELFEL_TILE_RUN; 0: one CTA per tile)
  int run_max = kTileRun;
  if (const char* e = getenv("ELFEL_TILE_RUN")) run_max = std::max(0, std::min(1 << 20, atoi(e)));
  if (run_max > 0) {
    std::vector<int2> runs;
    for (int64_t t = 0; t < nt;) {
      const TileHdr& h = tiles[t];
      int64_t u = t + 1;
      while (u < nt && u - t < run_max && (h.flags ? tiles[u].flags != 0 : (!tiles[u].flags && tiles[u].prog == h.prog)))
        ++u;
      runs.push_back(make_int2((int)t, (int)(u - t)));
      t = u;
    }
    T.nruns = (int64_t)runs.size();
    T.runlen = run_max;
    ELFEL_TRY(T.runs.alloc(c, runs.size()));
    ELFEL_CUDA(c, cudaMemcpyAsync(T.runs.p, runs.data(), sizeof(int2) * runs.size(), cudaMemcpyHostToDevice, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  T.maxblob = maxblob;
  T.maxnel = maxnel;
  T.nprograms = nprog;
  T.nfallback = nfb;
  T.built = 1;
  return ELFEL_OK;
}

static size_t tile_smem(const TilePlan& T) {
  return (size_t)T.maxblob + (size_t)T.maxnel * T.V * sizeof(double) + kTileMaxNz * sizeof(double);
}

static bool tile_runs_ok(const TilePlan& T) {
  return T.nruns > 0 && T.maxnel <= kRunThreads && T.V == kT6RTable && T.S == 21;
}

// Runs [r0, r0 + nr) of the plan's run kernel on stream s (T6 bases).
static int tile_reduce_runs(Ctx* c, const Pattern& P, const double* bases, double* vals, int64_t r0, int64_t nr,
                            cudaStream_t s) {
  const TilePlan& T = P.tiles;
  if (!T.built || !tile_runs_ok(T)) return fail(c, ELFEL_ERR_STATE, "tile runs without a T6 run plan");
  if (r0 < 0 || nr < 0 || r0 + nr > T.nruns) return fail(c, ELFEL_ERR_ARG, "tile runs outside the plan");
  if (nr == 0) return ELFEL_OK;
  const size_t sm = tile_smem(T);
  RecT6R r{bases};
  ELFEL_CUDA(c, cudaFuncSetAttribute(tile_run_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  tile_run_k<<<(unsigned)nr, kRunThreads, sm, s>>>(T.hdr.p, T.runs.p + r0, T.maxnel, T.maxblob, T.blob.p, P.cptr.p,
                                                   P.contrib.p, r, vals);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

int tile_reduce(Ctx* c, const Pattern& P, const double* src, int t6r_bases, double* vals) {
  const TilePlan& T = P.tiles;
  if (!T.built) return fail(c, ELFEL_ERR_STATE, "tile reduction without a plan");
  if (T.ntiles == 0) return ELFEL_OK;
  const size_t sm = tile_smem(T);
  if (t6r_bases) {
    if (T.V != kT6RTable || T.S != 21) return fail(c, ELFEL_ERR_STATE, "tile plan is not for T6 bases");
    RecT6R r{src};
    if (tile_runs_ok(T)) return tile_reduce_runs(c, P, src, vals, 0, T.nruns, c->stream);
    ELFEL_CUDA(c, cudaFuncSetAttribute(tile_reduce_k<RecT6R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    tile_reduce_k<RecT6R><<<(unsigned)T.ntiles, kRT, sm, c->stream>>>(T.hdr.p, T.maxnel, T.V, T.maxblob, T.blob.p,
                                                                       P.cptr.p, P.contrib.p, r, vals);
  } else {
    if (T.V != T.S) return fail(c, ELFEL_ERR_STATE, "tile plan is not for full records");
    RecFull r{src, T.S};
    ELFEL_CUDA(c, cudaFuncSetAttribute(tile_reduce_k<RecFull>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    tile_reduce_k<RecFull><<<(unsigned)T.ntiles, kRT, sm, c->stream>>>(T.hdr.p, T.maxnel, T.V, T.maxblob, T.blob.p,
                                                                        P.cptr.p, P.contrib.p, r, vals);
  }
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

}  // namespace elfel
