// Device construction of the CSC pattern and of the per-nonzero contributor
// lists (the "slot -> nonzero" map), with the semantics of
// SparseArrays.sparse(I, J, V, m, n) as called by finish! of
// SysmatAssemblerSparse (Elfel.jl src/Assemblers.jl:121-123):
//   * one slot per appended triplet, ordered as the assemble! calls append them;
//   * entries with equal (row, col) are summed in that slot order;
//   * explicitly assembled zeros stay in the pattern;
//   * rows ascend within each column.
//
// Steps (all deterministic; integer atomics only count and bucket):
//   1. column counts (one int32 atomic per column group in block mode, per
//      slot in COO mode)
//   2. exclusive scan -> column starts
//   3. bucket each slot's key (row << 32 | slot) into its column (one cursor
//      atomic per run of equal columns within a warp; the order inside a
//      column does not matter, the keys carry the slot)
//   4. sort each column's keys in registers (bitonic networks sized to the
//      column, 32-bit packed keys where the spans fit, 33-64 keys merged by
//      rank), count its distinct rows, write the storage index of every
//      contribution (contrib) in sorted order and the column's row starts
//   5. scan -> colptr; compact the row starts into rowval and the first
//      contribution of each nonzero (cptr)
//   6. (at a pattern's second value reduction) the contributor-count order
//      of each window of 128 nonzeros (window_order_k).
#include "pack32.cuh"
#include "sysmat.cuh"

namespace elfel {

constexpr int kSortThreads = 256;           // 8 warps
constexpr int kSortCap = 256;               // keys per warp sorted in shared memory

// Block mode: one thread per column group (one atomic per group instead of
// one per slot).  The row tables are the uploaded element DOF tables, range
// checked on upload; the column is checked here.
__global__ void count_groups_k(SlotGen g, int G, int64_t ngroups, int32_t* colcnt, int64_t ncol, int* bad) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ngroups; q += (int64_t)gridDim.x * blockDim.x) {
    int32_t c;
    int64_t s0;
    int len;
    const int32_t* rt;
    group_info(g, G, q, c, s0, len, rt);
    if (c < 0 || c >= ncol) {
      atomicExch(bad, 1);
      continue;
    }
    atomicAdd(&colcnt[c], len);
  }
}

__global__ void count_cols_k(SlotGen g, int64_t n, int32_t* colcnt, int64_t ncol, int64_t nrow, int* bad) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    int32_t r, c;
    int64_t st;
    slot_rc(g, s, r, c, st);
    if (r < 0 || r >= nrow || c < 0 || c >= ncol) {
      atomicExch(bad, 1);
      continue;
    }
    atomicAdd(&colcnt[c], 1);
  }
}

// Consecutive slots mostly share their column (a local column of an element
// matrix, a run of COO triplets): the lanes of a warp with equal columns in a
// row form a run whose first lane reserves the run's positions with one
// atomic and hands them out by shuffle.
__global__ void bucket_k(SlotGen g, int64_t n, const int64_t* colstart, int32_t* cursor, uint64_t* keys) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); s0 < n; s0 += stride) {
    const int64_t s = s0 + lane;
    const bool valid = s < n;
    int32_t r = 0, c = -1;
    int64_t st;
    if (valid) slot_rc(g, s, r, c, st);
    const int32_t cprev = __shfl_up_sync(0xffffffffu, c, 1);
    const bool head = valid && (lane == 0 || c != cprev);
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
    const int start = 31 - __clz(heads & upto);  // first lane of this lane's run
    int32_t base = 0;
    if (head) {
      const unsigned after = heads & ~upto;  // heads of later runs
      const int end = after ? __ffs(after) - 1 : 32 - __clz(vmask);
      base = atomicAdd(&cursor[c], end - lane);
    }
    base = __shfl_sync(0xffffffffu, base, valid ? start : 0);
    if (valid) keys[colstart[c] + base + (lane - start)] = ((uint64_t)(uint32_t)r << 32) | (uint64_t)(uint32_t)s;
  }
}

__device__ __forceinline__ void cmpswap(uint64_t* a, int64_t i, int64_t j) {
  uint64_t x = a[i], y = a[j];
  if (x > y) {
    a[i] = y;
    a[j] = x;
  }
}

// Bitonic network in its "flip" form: every comparator puts the smaller key at
// the lower index, so any length n sorts correctly when comparators that reach
// past n are skipped (those positions behave as +infinity).  One warp.  The
// sizes are powers of two below 2^31 (a column holds fewer than 2^31 slots),
// so block and offset come from 32-bit shifts and masks.
__device__ void warp_sort(uint64_t* a, int n, int lane) {
  if (n < 2) return;
  const unsigned un = (unsigned)n;
  int lg = 0;
  while ((1u << lg) < un) ++lg;
  const unsigned half_pairs = 1u << (lg - 1);
  for (int ls = 1; ls <= lg; ++ls) {  // size = 2^ls, h = 2^(ls - 1)
    const int lh = ls - 1;
    const unsigned size = 1u << ls, h = 1u << lh;
    for (unsigned p = lane; p < half_pairs; p += 32) {
      const unsigned blk = p >> lh, off = p & (h - 1);
      const unsigned i = blk * size + off;
      const unsigned j = blk * size + size - 1 - off;
      if (j < un) cmpswap(a, i, j);
    }
    __syncwarp();
    for (int lst = lh - 1; lst >= 0; --lst) {  // stride = 2^lst
      const unsigned stride = 1u << lst;
      for (unsigned p = lane; p < half_pairs; p += 32) {
        const unsigned blk = p >> lst, off = p & (stride - 1);
        const unsigned i = (blk << (lst + 1)) + off;
        const unsigned j = i + stride;
        if (j < un) cmpswap(a, i, j);
      }
      __syncwarp();
    }
  }
}

// Register-resident bitonic sort of P <= 32 keys, one per lane: lanes 0..P-1
// end ascending (every group of P lanes is sorted, in alternating
// directions); shuffles exchange the partners.  Unused lanes hold ~0.
template <int P, typename K>
__device__ __forceinline__ K reg_sort(K v, int lane) {
#pragma unroll
  for (int k = 2; k <= P; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const K o = __shfl_xor_sync(0xffffffffu, v, j);
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      v = keep_min ? (v < o ? v : o) : (v < o ? o : v);
    }
  }
  return v;
}

// Number of keys of a sequence sorted ascending across the warp's lanes
// (one per lane, padding ~0) that are below x (keys are distinct): a binary
// search whose probes are per-lane shuffles.
template <typename K>
__device__ __forceinline__ int count_below(K seq, K x) {
  int pos = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1)
    if (__shfl_sync(0xffffffffu, seq, pos + step - 1) < x) pos += step;
  if (__shfl_sync(0xffffffffu, seq, pos) < x) ++pos;
  return pos;
}

__device__ __forceinline__ int bit_length(uint32_t x) { return x ? 32 - __clz((int)x) : 0; }

// A column whose row and slot spans fit in 31 bits together is sorted on
// 32-bit packed keys (pack32.cuh): a compare-exchange stage of the register
// sorts then costs half the instructions of the 64-bit one.  The packing of
// the keys of the whole warp (valid keys: lo <= hi per field; lanes without
// keys pass lo = ~0u, hi = 0); false when it does not fit.
__device__ __forceinline__ bool pack_warp(uint32_t rlo, uint32_t rhi, uint32_t slo, uint32_t shi, Pack32* p) {
  const uint32_t rmin = __reduce_min_sync(0xffffffffu, rlo), rmax = __reduce_max_sync(0xffffffffu, rhi);
  const uint32_t smin = __reduce_min_sync(0xffffffffu, slo), smax = __reduce_max_sync(0xffffffffu, shi);
  if (rmax < rmin || smax < smin) return false;
  const int sb = bit_length(smax - smin);
  if (bit_length(rmax - rmin) + sb > 31) return false;
  *p = Pack32{rmin, smin, sb};
  return true;
}

// The same for each half warp separately (xor partners below 16).
__device__ __forceinline__ bool pack_half(uint32_t rlo, uint32_t rhi, uint32_t slo, uint32_t shi, Pack32* p) {
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    rlo = min(rlo, __shfl_xor_sync(0xffffffffu, rlo, o));
    rhi = max(rhi, __shfl_xor_sync(0xffffffffu, rhi, o));
    slo = min(slo, __shfl_xor_sync(0xffffffffu, slo, o));
    shi = max(shi, __shfl_xor_sync(0xffffffffu, shi, o));
  }
  if (rhi < rlo || shi < slo) return false;
  const int sb = bit_length(shi - slo);
  if (bit_length(rhi - rlo) + sb > 31) return false;
  *p = Pack32{rlo, slo, sb};
  return true;
}

// Output of a sorted column: each key's storage index goes to contrib[b + t]
// (t = its place in the column), and each key that starts a row (its
// predecessor has another row) to nzkey[b + i] as (row << 32 | b + t), i =
// the number of rows before it in the column.  compact_k moves the latter to
// rowval / cptr once the column's first nonzero is known.
struct ColOut {
  int32_t* contrib;
  uint64_t* nzkey;
};

__device__ __forceinline__ void put_key(const SlotGen& g, const ColOut& o, int64_t b, uint64_t key, int t, bool first,
                                        int li) {
  o.contrib[b + t] = (int32_t)slot_store(g, (int64_t)(key & 0xffffffffull));
  if (first) o.nzkey[b + li] = (key & 0xffffffff00000000ull) | (uint64_t)(uint32_t)(b + t);
}

// Sort 32 < n <= 64 keys (keys[b + lane], keys[b + 32 + lane]) by merging:
// the first 32 and the other n - 32 are sorted in registers separately, each
// key's place is its index plus the number of keys of the other sequence
// below it; the keys are placed in sh and read back in order.
__device__ __forceinline__ void sort_column_merge(const SlotGen& g, const ColOut& o, int64_t b, int n,
                                                  const uint64_t* keys, int32_t* cnt_out, uint64_t* sh, int lane) {
  uint64_t v0 = keys[b + lane];
  uint64_t v1 = lane + 32 < n ? keys[b + lane + 32] : ~0ull;
  const int m = n - 32;
  const bool has1 = lane < m;
  const uint32_t r0v = (uint32_t)(v0 >> 32), s0v = (uint32_t)v0;
  const uint32_t r1v = (uint32_t)(v1 >> 32), s1v = (uint32_t)v1;
  Pack32 pk;
  if (pack_warp(has1 ? min(r0v, r1v) : r0v, has1 ? max(r0v, r1v) : r0v, has1 ? min(s0v, s1v) : s0v,
                has1 ? max(s0v, s1v) : s0v, &pk)) {
    uint32_t k0 = pack32(v0, pk), k1 = has1 ? pack32(v1, pk) : ~0u;
    k0 = reg_sort<32>(k0, lane);
    if (m > 16) k1 = reg_sort<32>(k1, lane);
    else if (m > 8) k1 = reg_sort<16>(k1, lane);
    else if (m > 4) k1 = reg_sort<8>(k1, lane);
    else if (m > 1) k1 = reg_sort<4>(k1, lane);
    const int r0 = lane + count_below(k1, k0);
    const int r1 = lane + count_below(k0, k1);
    sh[r0] = unpack32(k0, pk);
    if (has1) sh[r1] = unpack32(k1, pk);
  } else {
    v0 = reg_sort<32>(v0, lane);
    if (m > 16) v1 = reg_sort<32>(v1, lane);
    else if (m > 8) v1 = reg_sort<16>(v1, lane);
    else if (m > 4) v1 = reg_sort<8>(v1, lane);
    else if (m > 1) v1 = reg_sort<4>(v1, lane);
    const int r0 = lane + count_below(v1, v0);
    const int r1 = lane + count_below(v0, v1);
    sh[r0] = v0;
    if (has1) sh[r1] = v1;
  }
  __syncwarp();
  const uint64_t s0 = sh[lane], s1 = lane + 32 < n ? sh[lane + 32] : ~0ull;
  const uint64_t p0 = __shfl_up_sync(0xffffffffu, s0, 1);
  const uint64_t last0 = __shfl_sync(0xffffffffu, s0, 31);
  uint64_t p1 = __shfl_up_sync(0xffffffffu, s1, 1);
  if (lane == 0) p1 = last0;
  const bool f0 = lane == 0 || (s0 >> 32) != (p0 >> 32);
  const bool f1 = lane + 32 < n && (s1 >> 32) != (p1 >> 32);
  const unsigned m0 = __ballot_sync(0xffffffffu, f0), m1 = __ballot_sync(0xffffffffu, f1);
  const unsigned below = (1u << lane) - 1u;
  put_key(g, o, b, s0, lane, f0, __popc(m0 & below));
  if (lane + 32 < n) put_key(g, o, b, s1, lane + 32, f1, __popc(m0) + __popc(m1 & below));
  if (lane == 0) *cnt_out = __popc(m0) + __popc(m1);
  __syncwarp();  // sh is reused by the warp's next column
}

// Sort one column's keys by (row, slot), write its output (ColOut) and its
// number of distinct rows (one warp).  Columns of up to 32 keys are sorted in
// registers, up to 64 by sort_column_merge; longer ones with the bitonic
// network in shared memory (up to kSortCap keys, in sh) or in place in global
// memory.
__device__ void sort_column(const SlotGen& g, const ColOut& o, int64_t b, int n, uint64_t* keys, int32_t* cnt_out,
                            uint64_t* sh, int lane) {
  const unsigned below = (1u << lane) - 1u;
  if (n <= 32) {
    const bool has = lane < n;
    uint64_t v = has ? keys[b + lane] : ~0ull;
    Pack32 pk;
    const uint32_t rv = (uint32_t)(v >> 32), sv = (uint32_t)v;
    if (n > 1 && pack_warp(has ? rv : ~0u, has ? rv : 0u, has ? sv : ~0u, has ? sv : 0u, &pk)) {
      uint32_t k = has ? pack32(v, pk) : ~0u;
      if (n > 16) k = reg_sort<32>(k, lane);
      else if (n > 8) k = reg_sort<16>(k, lane);
      else if (n > 4) k = reg_sort<8>(k, lane);
      else k = reg_sort<4>(k, lane);
      v = has ? unpack32(k, pk) : ~0ull;
    } else {
      if (n > 16) v = reg_sort<32>(v, lane);
      else if (n > 8) v = reg_sort<16>(v, lane);
      else if (n > 4) v = reg_sort<8>(v, lane);
      else if (n > 1) v = reg_sort<4>(v, lane);
    }
    // distinct rows: a key starts a row when its predecessor has another row
    const uint64_t pv = __shfl_up_sync(0xffffffffu, v, 1);
    const bool first = lane < n && (lane == 0 || (v >> 32) != (pv >> 32));
    const unsigned m = __ballot_sync(0xffffffffu, first);
    if (lane < n) put_key(g, o, b, v, lane, first, __popc(m & below));
    if (lane == 0) *cnt_out = __popc(m);
    return;
  }
  if (n <= 64) {
    sort_column_merge(g, o, b, n, keys, cnt_out, sh, lane);
    return;
  }
  uint64_t* a;
  if (n <= kSortCap) {
    for (int t = lane; t < n; t += 32) sh[t] = keys[b + t];
    __syncwarp();
    a = sh;
  } else {
    a = keys + b;  // long column: sort in place in global memory
  }
  warp_sort(a, n, lane);
  int32_t cnt = 0;
  for (int t0 = 0; t0 < n; t0 += 32) {
    const int t = t0 + lane;
    bool first = false;
    uint64_t key = 0;
    if (t < n) {
      key = a[t];
      first = (t == 0) || ((key >> 32) != (a[t - 1] >> 32));
    }
    const unsigned m = __ballot_sync(0xffffffffu, first);
    if (t < n) put_key(g, o, b, key, t, first, cnt + __popc(m & below));
    cnt += __popc(m);
  }
  if (lane == 0) *cnt_out = cnt;
  __syncwarp();
}

// A warp takes four consecutive columns.  When each has at most 8 keys (the
// rhs pattern, where a column holds a node's element contributions), the
// four are sorted at once, one per group of 8 lanes; when each has at most
// 16 (T6 midside columns), two at a time; otherwise one after the other by
// the whole warp.
constexpr int kColsPerWarp = 4;

__global__ void __launch_bounds__(kSortThreads) sort_cols_k(SlotGen g, ColOut o, const int64_t* colstart,
                                                           int64_t ncol, uint64_t* keys, int32_t* nnzcnt) {
  __shared__ uint64_t sh[kSortThreads / 32][kSortCap];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int grp = lane >> 3, gl = lane & 7;
  const unsigned below = (1u << lane) - 1u;
  const int64_t warps = (int64_t)gridDim.x * (kSortThreads / 32);
  for (int64_t c0 = ((int64_t)blockIdx.x * (kSortThreads / 32) + wid) * kColsPerWarp; c0 < ncol;
       c0 += warps * kColsPerWarp) {
    const int64_t cg = c0 + grp;
    int64_t bg = 0;
    int ng = 0;
    if (cg < ncol) {
      bg = colstart[cg];
      ng = (int)(colstart[cg + 1] - bg);
    }
    if (__all_sync(0xffffffffu, ng <= 8)) {
      uint64_t v = gl < ng ? keys[bg + gl] : ~0ull;
      v = reg_sort<8>(v, gl);  // partners lane ^ j (j < 8) stay inside the group
      const uint64_t pv = __shfl_up_sync(0xffffffffu, v, 1, 8);
      const bool first = gl < ng && (gl == 0 || (v >> 32) != (pv >> 32));
      const unsigned group = 0xffu << (grp * 8);
      const unsigned m = __ballot_sync(0xffffffffu, first) & group;
      if (gl < ng) put_key(g, o, bg, v, gl, first, __popc(m & below));
      if (gl == 0 && cg < ncol) nnzcnt[cg] = __popc(m);
      continue;
    }
    if (__all_sync(0xffffffffu, ng <= 16)) {
      // two columns at a time, one per half warp (T6 midside columns: 12 keys)
      const int h = lane >> 4, hl = lane & 15;
      const unsigned half = 0xffffu << (h * 16);
#pragma unroll
      for (int r = 0; r < kColsPerWarp / 2; ++r) {
        const int q = 2 * r + h;
        const int64_t b = __shfl_sync(0xffffffffu, bg, q * 8);
        const int n = __shfl_sync(0xffffffffu, ng, q * 8);
        const bool has = hl < n;
        uint64_t v = has ? keys[b + hl] : ~0ull;
        const uint32_t rv = (uint32_t)(v >> 32), sv = (uint32_t)v;
        Pack32 pk;
        // partners lane ^ j (j < 16) stay inside the half; both halves take
        // the same branch only when both packings fit
        const bool fit = pack_half(has ? rv : ~0u, has ? rv : 0u, has ? sv : ~0u, has ? sv : 0u, &pk);
        if (__all_sync(0xffffffffu, fit || n <= 1)) {
          uint32_t k = has && n > 1 ? pack32(v, pk) : ~0u;
          k = reg_sort<16>(k, hl);
          if (n > 1) v = has ? unpack32(k, pk) : ~0ull;
        } else {
          v = reg_sort<16>(v, hl);
        }
        const uint64_t pv = __shfl_up_sync(0xffffffffu, v, 1, 16);
        const bool first = hl < n && (hl == 0 || (v >> 32) != (pv >> 32));
        const unsigned m = __ballot_sync(0xffffffffu, first) & half;
        if (hl < n) put_key(g, o, b, v, hl, first, __popc(m & below));
        if (hl == 0 && c0 + q < ncol) nnzcnt[c0 + q] = __popc(m);
      }
      continue;
    }
    for (int q = 0; q < kColsPerWarp; ++q) {
      const int64_t col = c0 + q;
      if (col >= ncol) break;
      const int64_t b = colstart[col];
      sort_column(g, o, b, (int)(colstart[col + 1] - b), keys, nnzcnt + col, sh[wid], lane);
    }
  }
}

// rowval / cptr of every column from its row starts (ColOut.nzkey): one half
// warp per column.
__global__ void compact_k(const int64_t* __restrict__ colstart, const int64_t* __restrict__ colptr, int64_t ncol,
                          const uint64_t* __restrict__ nzkey, int32_t* __restrict__ rowval,
                          int32_t* __restrict__ cptr) {
  const int hl = threadIdx.x & 15;
  const int64_t halves = (int64_t)gridDim.x * (blockDim.x / 16);
  for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 4; c < ncol; c += halves) {
    const int64_t k0 = colptr[c], cnt = colptr[c + 1] - k0, b = colstart[c];
    for (int64_t i = hl; i < cnt; i += 16) {
      const uint64_t v = nzkey[b + i];
      rowval[k0 + i] = (int32_t)(v >> 32);
      cptr[k0 + i] = (int32_t)(uint32_t)v;
    }
  }
}

__global__ void set_last_k(int32_t* cptr, int64_t nnz, int64_t total) { cptr[nnz] = (int32_t)total; }

// For every window of kReduceWindow nonzeros (one warp each): the window's
// nonzeros ordered by contributor count (counts of 8 and more together), ties
// by position -- a stable bucket order; perm[w * kReduceWindow + rank] =
// position in the window.  Positions past the last nonzero sort last.  The
// ranks come from one ballot per bucket and round: rank = items in smaller
// buckets + items of the same bucket in earlier rounds or lower lanes.
constexpr int kOrderBuckets = 8;

__global__ void window_order_k(const int32_t* __restrict__ cptr, int64_t nnz, uint8_t* __restrict__ perm) {
  constexpr int R = kReduceWindow / 32;
  const int lane = threadIdx.x & 31;
  const unsigned lower = (1u << lane) - 1u;
  const int64_t nwin = (nnz + kReduceWindow - 1) / kReduceWindow;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); w < nwin; w += warps) {
    const int64_t base = w * kReduceWindow;
    const int n = (int)min((int64_t)kReduceWindow, nnz - base);
    int v[R], rank[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int j = r * 32 + lane;
      v[r] = kOrderBuckets;  // padding: after every bucket
      if (j < n) {
        const int c = cptr[base + j + 1] - cptr[base + j];
        v[r] = (c < 1 ? 1 : (c > kOrderBuckets ? kOrderBuckets : c)) - 1;
      }
      rank[r] = 0;
    }
    int start = 0;
#pragma unroll
    for (int bkt = 0; bkt <= kOrderBuckets; ++bkt) {
      int before = start;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const unsigned m = __ballot_sync(0xffffffffu, v[r] == bkt);
        if (v[r] == bkt) rank[r] = before + __popc(m & lower);
        before += __popc(m);
      }
      start = before;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) perm[base + rank[r]] = (uint8_t)(r * 32 + lane);
  }
}

int build_pattern(Ctx* c, const SlotGen& g0, int64_t nrow, int64_t ncol, Pattern* P) {
  SlotGen g = g0;
  g.prepare();
  P->release(c);
  const int64_t M = g.total();
  if (M >= (int64_t)0x7fffffff)
    return fail(c, ELFEL_ERR_ARG, "too many assembled entries (%lld): the device pattern holds < 2^31", (long long)M);
  if (nrow >= (int64_t)0x7fffffff || ncol >= (int64_t)0x7fffffff)
    return fail(c, ELFEL_ERR_ARG, "matrix dimension >= 2^31");
  P->nrow = nrow;
  P->ncol = ncol;
  P->nslots = M;
  cudaStream_t st = c->stream;
  DBuf<int32_t> colcnt, cursor;
  DBuf<int64_t> colstart;
  DBuf<uint64_t> keys;
  DBuf<int> bad;
  ELFEL_TRY(colcnt.alloc(c, (size_t)ncol + 1));
  ELFEL_TRY(cursor.alloc(c, (size_t)ncol + 1));
  ELFEL_TRY(colstart.alloc(c, (size_t)ncol + 1));
  ELFEL_TRY(bad.alloc(c, 1));
  ELFEL_CUDA(c, cudaMemsetAsync(colcnt.p, 0, sizeof(int32_t) * (ncol + 1), st));
  ELFEL_CUDA(c, cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * (ncol + 1), st));
  ELFEL_CUDA(c, cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  const unsigned gs = grid_for(M, 256, (int64_t)c->sm_count * 16);
  const int G = groups_per_elem(g);
  const int64_t ngroups = g.nblocks ? g.nel * (int64_t)G : 0;
  if (M > 0) {
    if (g.nblocks)
      count_groups_k<<<grid_for(ngroups, 256, (int64_t)c->sm_count * 16), 256, 0, st>>>(g, G, ngroups, colcnt.p,
                                                                                        ncol, bad.p);
    else
      count_cols_k<<<gs, 256, 0, st>>>(g, M, colcnt.p, ncol, nrow, bad.p);
    ELFEL_LAUNCH_CHECK(c);
  }
  int hbad = 0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  ELFEL_CUDA(c, cudaStreamSynchronize(st));
  if (hbad) return fail(c, ELFEL_ERR_ARG, "assembled row or column number out of range (1..%lld, 1..%lld)",
                        (long long)nrow, (long long)ncol);
  ELFEL_TRY(scan_counts_i32(c, colcnt.p, ncol, colstart.p));
  ELFEL_TRY(keys.alloc(c, (size_t)(M > 0 ? M : 1)));
  if (M > 0) {
    bucket_k<<<gs, 256, 0, st>>>(g, M, colstart.p, cursor.p, keys.p);
    ELFEL_LAUNCH_CHECK(c);
  }
  cursor.release(c);
  // sort + distinct counts (reuse colcnt as per-column nonzero counts)
  const unsigned gsort = grid_for((ncol + kColsPerWarp - 1) / kColsPerWarp, kSortThreads / 32,
                                  (int64_t)c->sm_count * 32);
  DBuf<uint64_t> nzkey;  // row starts of each column (ColOut), compacted after the scan
  ELFEL_TRY(nzkey.alloc(c, (size_t)(M > 0 ? M : 1)));
  ELFEL_TRY(P->contrib.alloc(c, (size_t)(M > 0 ? M : 1)));
  if (ncol > 0) {
    sort_cols_k<<<gsort, kSortThreads, 0, st>>>(g, ColOut{P->contrib.p, nzkey.p}, colstart.p, ncol, keys.p,
                                               colcnt.p);
    ELFEL_LAUNCH_CHECK(c);
  }
  ELFEL_TRY(P->colptr.alloc(c, (size_t)ncol + 1));
  ELFEL_TRY(scan_counts_i32(c, colcnt.p, ncol, P->colptr.p));
  int64_t nnz = 0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&nnz, P->colptr.p + ncol, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  ELFEL_CUDA(c, cudaStreamSynchronize(st));
  P->nnz = nnz;
  ELFEL_TRY(P->rowval.alloc(c, (size_t)(nnz > 0 ? nnz : 1)));
  ELFEL_TRY(P->cptr.alloc(c, (size_t)nnz + 1));
  if (ncol > 0) {
    compact_k<<<grid_for(ncol, 16, (int64_t)c->sm_count * 32), 256, 0, st>>>(colstart.p, P->colptr.p, ncol,
                                                                            nzkey.p, P->rowval.p, P->cptr.p);
    ELFEL_LAUNCH_CHECK(c);
  }
  nzkey.release(c);
  set_last_k<<<1, 1, 0, st>>>(P->cptr.p, nnz, M);
  ELFEL_LAUNCH_CHECK(c);
  keys.release(c);
  colcnt.release(c);
  colstart.release(c);
  bad.release(c);
  return ELFEL_OK;
}

// One thread per nonzero; its contributions are summed left to right, in the
// order the reference's sparse() adds duplicates.
// Each thread reduces kReduceItems nonzeros (k, k + stride, ...) with their
// loads interleaved, so that several independent load chains (cptr ->
// contrib -> record) are in flight per thread; every nonzero still adds its
// contributions in slot order.
constexpr int kReduceItems = 4;

__global__ void reduce_k(const int32_t* __restrict__ cptr, const int32_t* __restrict__ contrib,
                         const double* __restrict__ store, int64_t nnz, double* __restrict__ out) {
  constexpr int R = kReduceItems;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k0 < nnz; k0 += R * stride) {
    int32_t b[R], e[R];
    double s[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int64_t k = k0 + i * stride;
      b[i] = 0;
      e[i] = 0;
      if (k < nnz) {
        b[i] = cptr[k];
        e[i] = cptr[k + 1];
      }
    }
#pragma unroll
    for (int i = 0; i < R; ++i) s[i] = b[i] < e[i] ? store[contrib[b[i]]] : 0.0;
#pragma unroll
    for (int i = 0; i < R; ++i)
      if (b[i] + 1 < e[i]) s[i] += store[contrib[b[i] + 1]];
#pragma unroll
    for (int i = 0; i < R; ++i)
      for (int32_t t = b[i] + 2; t < e[i]; ++t) s[i] += store[contrib[t]];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int64_t k = k0 + i * stride;
      if (k < nnz) out[k] = s[i];
    }
  }
}

// One warp per window of kReduceWindow nonzeros, four rounds of 32 lanes in
// the window's contributor-count order: the lanes of a round have similar
// counts, so a round issues about as many FP64 adds as its nonzeros need
// (every warp-level FP64 instruction costs the SM's FP64 pipe the same time
// however few of its lanes are active).  Each nonzero still adds its
// contributions in slot order, and the window's values are written inside
// its own 1 KB of the output.
__global__ void __launch_bounds__(256) reduce_win_k(const int32_t* __restrict__ cptr,
                                                   const int32_t* __restrict__ contrib,
                                                   const uint8_t* __restrict__ perm,
                                                   const double* __restrict__ store, int64_t nnz,
                                                   double* __restrict__ out) {
  constexpr int R = kReduceWindow / 32;
  const int lane = threadIdx.x & 31;
  const int64_t nwin = (nnz + kReduceWindow - 1) / kReduceWindow;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); w < nwin; w += warps) {
    const int64_t base = w * kReduceWindow;
    const int n = (int)min((int64_t)kReduceWindow, nnz - base);
    int j[R];
    int32_t b[R], e[R];
    double s[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      j[r] = perm[base + r * 32 + lane];
      b[r] = 0;
      e[r] = 0;
      if (j[r] < n) {
        b[r] = cptr[base + j[r]];
        e[r] = cptr[base + j[r] + 1];
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) s[r] = b[r] < e[r] ? store[contrib[b[r]]] : 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (b[r] + 1 < e[r]) s[r] += store[contrib[b[r] + 1]];
#pragma unroll
    for (int r = 0; r < R; ++r)
      for (int32_t t = b[r] + 2; t < e[r]; ++t) s[r] += store[contrib[t]];
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (j[r] < n) out[base + j[r]] = s[r];
  }
}

// Many reductions in one launch: CTA b serves job k with jobs[k].blk0 <= b <
// jobs[k+1].blk0, items (b - blk0) * blockDim.x onwards.  A job with colptr
// reduces a 1 x n pattern into a dense vector (the rhs), else the nnz values.
// Each item adds its contributions in slot order, as reduce_k.
__global__ void reduce_batch_k(const RedJob* __restrict__ jobs, int njobs) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].blk0 <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
  }
  const RedJob J = jobs[lo];
  const int64_t k = ((int64_t)blockIdx.x - J.blk0) * blockDim.x + threadIdx.x;
  if (k >= J.n) return;
  int64_t slot = k;
  if (J.colptr) {
    const int64_t k0 = J.colptr[k], k1 = J.colptr[k + 1];
    if (k1 == k0) {
      J.out[k] = 0.0;
      return;
    }
    slot = k0;
  }
  const int32_t b = J.cptr[slot], e = J.cptr[slot + 1];
  double s = J.store[J.contrib[b]];
  if (J.colptr) s = __dadd_rn(0.0, s);  // a vector starts from a zeroed one (SysvecAssembler)
  for (int32_t t = b + 1; t < e; ++t) s += J.store[J.contrib[t]];
  J.out[k] = s;
}

int reduce_batch(Ctx* c, const RedJob* jobs_dev, int njobs, int64_t blocks) {
  if (njobs == 0 || blocks == 0) return ELFEL_OK;
  if (blocks > 0x7fffffff) return fail(c, ELFEL_ERR_ARG, "batched reduction: too many items");
  reduce_batch_k<<<(unsigned)blocks, kRedJobThreads, 0, c->stream>>>(jobs_dev, njobs);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

int reduce_values(Ctx* c, Pattern& P, const double* store, double* vals_out) {
  if (P.nnz == 0) return ELFEL_OK;
  // The count order (window_order_k) pays for itself from a pattern's second
  // reduction on; a pattern reduced once (an end-to-end call) does without it.
  // Both kernels add every nonzero's contributions in slot order: same bits.
  // 1 x n patterns (vectors) are reduced by reduce_dense.
  if (!P.perm.p && P.reductions >= 1 && P.nrow > 1) {
    const int64_t nwin = (P.nnz + kReduceWindow - 1) / kReduceWindow;
    ELFEL_TRY(P.perm.alloc(c, (size_t)(nwin * kReduceWindow)));
    window_order_k<<<grid_for(nwin, 8, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(P.cptr.p, P.nnz, P.perm.p);
    ELFEL_LAUNCH_CHECK(c);
  }
  P.reductions++;
  if (P.perm.p) {
    const int64_t nwin = (P.nnz + kReduceWindow - 1) / kReduceWindow;
    reduce_win_k<<<grid_for(nwin, 8, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
        P.cptr.p, P.contrib.p, P.perm.p, store, P.nnz, vals_out);
  } else {
    reduce_k<<<grid_for(P.nnz, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(P.cptr.p, P.contrib.p, store,
                                                                                     P.nnz, vals_out);
  }
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

__global__ void to_index32_k(const int64_t* src, int64_t n, int64_t limit, int32_t* dst, int* bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = src[i];
    if (v < 1 || v > limit) {
      atomicExch(bad, 1);
      dst[i] = 0;
    } else {
      dst[i] = (int32_t)(v - 1);
    }
  }
}

// The same conversion reading the (device-readable) host array directly:
// four independent loads per thread keep enough bytes in flight over the
// host link with a small grid, which leaves most of the SMs to the work on
// other streams.
__global__ void to_index32_host_k(const int64_t* __restrict__ src, int64_t n, int64_t limit, int32_t* __restrict__ dst,
                                  int* __restrict__ bad) {
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += U * stride) {
    int64_t v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = i0 + u * stride < n ? src[i0 + u * stride] : 1;
    bool b = false;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool out = v[u] < 1 || v[u] > limit;
      b |= out;
      if (i0 + u * stride < n) dst[i0 + u * stride] = out ? 0 : (int32_t)(v[u] - 1);
    }
    if (b) atomicExch(bad, 1);
  }
}

__global__ void copy_host_f64_k(const double* __restrict__ src, int64_t n, double* __restrict__ dst) {
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += U * stride) {
    double v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = i0 + u * stride < n ? src[i0 + u * stride] : 0.0;
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (i0 + u * stride < n) dst[i0 + u * stride] = v[u];
  }
}

int to_index32_direct(Ctx* c, cudaStream_t st, const int64_t* src, int64_t n, int64_t limit, int32_t* dst, int* bad) {
  if (n == 0) return ELFEL_OK;
  to_index32_host_k<<<grid_for(n, 256 * 4, (int64_t)c->sm_count * 2), 256, 0, st>>>(src, n, limit, dst, bad);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

int copy_host_f64(Ctx* c, cudaStream_t st, const double* src, int pinned, int64_t n, double* dst) {
  if (n == 0) return ELFEL_OK;
  if (pinned) {
    ELFEL_CUDA(c, cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    return ELFEL_OK;
  }
  copy_host_f64_k<<<grid_for(n, 256 * 4, (int64_t)c->sm_count * 2), 256, 0, st>>>(src, n, dst);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

int to_index32(Ctx* c, const int64_t* src_host, int64_t n, int64_t limit, DBuf<int32_t>* dst, const char* what) {
  ELFEL_TRY(dst->alloc(c, (size_t)(n > 0 ? n : 1)));
  if (n == 0) return ELFEL_OK;
  DBuf<int64_t> tmp;
  DBuf<int> bad;
  ELFEL_TRY(tmp.alloc(c, (size_t)n));
  ELFEL_TRY(bad.alloc(c, 1));
  ELFEL_CUDA(c, cudaMemsetAsync(bad.p, 0, sizeof(int), c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(tmp.p, src_host, sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->stream));
  to_index32_k<<<grid_for(n, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(tmp.p, n, limit, dst->p, bad.p);
  ELFEL_LAUNCH_CHECK(c);
  int hbad = 0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  tmp.release(c);
  bad.release(c);
  if (hbad) return fail(c, ELFEL_ERR_ARG, "%s: entry outside 1..%lld", what, (long long)limit);
  return ELFEL_OK;
}

}  // namespace elfel
