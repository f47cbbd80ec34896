// Allocation-free form of the device vector assembly (elfel_sysvec_assemble).
//
// Some callers cannot allocate device memory at the point where they assemble:
// a host program that hands the library only memory it manages itself (a pool
// owned by another runtime), or a loop that must not call cudaMalloc because
// allocation synchronises the device and takes unbounded time.  This entry
// point takes device pointers for its inputs and output and keeps all of its
// scratch in one file-scope device array of fixed size (kNaBytes, about 16 MB,
// held by every GPU that loads the library until the process exits).
//
// Result: out[r] = +0 plus vals[s] over the entries s with rows[s] == r + 1,
// added in increasing s -- the same order, hence the same bits (signed zeros
// included), as elfel_sysvec_assemble and the reference's SysvecAssembler.
// A row number outside 1..nrow fails the call and leaves out unchanged.
//
// Steps: clear counters, count per row (integer atomics), exclusive scan,
// bucket entry indices per row, sort each row's indices (one warp per row),
// add the values in that order.
#include <mutex>

#include "common.cuh"

namespace {

constexpr int64_t kNaMaxRows = ELFEL_NOALLOC_MAX_ROWS;
constexpr int64_t kNaMaxEntries = ELFEL_NOALLOC_MAX_ENTRIES;
constexpr int kNaScanBlock = 512;
constexpr int kNaScanItems = 8;
constexpr int64_t kNaTile = kNaScanBlock * kNaScanItems;
constexpr int64_t kNaTiles = (kNaMaxRows + kNaTile - 1) / kNaTile;

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
// byte offsets of the scratch areas
constexpr size_t kOffCounts = 0;
constexpr size_t kOffCursor = kOffCounts + align256(sizeof(int32_t) * kNaMaxRows);
constexpr size_t kOffOffsets = kOffCursor + align256(sizeof(int32_t) * kNaMaxRows);
constexpr size_t kOffTileTot = kOffOffsets + align256(sizeof(int64_t) * (kNaMaxRows + 1));
constexpr size_t kOffTileOff = kOffTileTot + align256(sizeof(int64_t) * kNaTiles);
constexpr size_t kOffOrder = kOffTileOff + align256(sizeof(int64_t) * (kNaTiles + 1));
constexpr size_t kOffFlag = kOffOrder + align256(sizeof(uint32_t) * kNaMaxEntries);
constexpr size_t kNaBytes = kOffFlag + 256;

// The scratch.  Host code must not pass this name to a kernel: on the host it
// is only a stand-in symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_na_scratch[kNaBytes];

struct View {
  int32_t* counts;
  int32_t* cursor;
  int64_t* offsets;
  int64_t* tile_tot;
  int64_t* tile_off;
  uint32_t* order;
  int* bad;
};

View carve(void* base) {
  unsigned char* b = static_cast<unsigned char*>(base);
  return View{reinterpret_cast<int32_t*>(b + kOffCounts), reinterpret_cast<int32_t*>(b + kOffCursor),
              reinterpret_cast<int64_t*>(b + kOffOffsets), reinterpret_cast<int64_t*>(b + kOffTileTot),
              reinterpret_cast<int64_t*>(b + kOffTileOff), reinterpret_cast<uint32_t*>(b + kOffOrder),
              reinterpret_cast<int*>(b + kOffFlag)};
}

// device address of g_na_scratch per device, set once with that device current
constexpr int kMaxDevices = 64;
void* g_na_addr[kMaxDevices] = {};
std::mutex g_na_mutex;

__global__ void na_clear_k(View v, int64_t nrow) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrow; i += (int64_t)gridDim.x * blockDim.x) {
    v.counts[i] = 0;
    v.cursor[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *v.bad = 0;
}

__global__ void na_count_k(View v, const int64_t* __restrict__ rows, int64_t n, int64_t nrow) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = rows[s] - 1;
    if (r < 0 || r >= nrow) {
      atomicExch(v.bad, 1);
      continue;
    }
    atomicAdd(&v.counts[r], 1);
  }
}

// tile totals of the counts
__global__ void na_tile_tot_k(View v, int64_t nrow) {
  __shared__ int64_t sh[kNaScanBlock / 32];
  const int64_t base = (int64_t)blockIdx.x * kNaTile;
  int64_t s = 0;
  for (int k = 0; k < kNaScanItems; ++k) {
    const int64_t i = base + (int64_t)k * kNaScanBlock + threadIdx.x;
    if (i < nrow) s += v.counts[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < kNaScanBlock / 32; ++w) t += sh[w];
    v.tile_tot[blockIdx.x] = t;
  }
}

// exclusive scan of the (at most kNaTiles) tile totals: one thread, in order
__global__ void na_tile_scan_k(View v, int64_t ntiles) {
  int64_t run = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    v.tile_off[t] = run;
    run += v.tile_tot[t];
  }
  v.tile_off[ntiles] = run;
}

// exclusive scan inside each tile plus the tile offset -> offsets[0..nrow]
__global__ void na_tile_k(View v, int64_t nrow, int64_t ntiles) {
  __shared__ int64_t warp_tot[kNaScanBlock / 32];
  const int64_t base = (int64_t)blockIdx.x * kNaTile + (int64_t)threadIdx.x * kNaScanItems;
  int64_t vals[kNaScanItems];
  int64_t run = 0;
  for (int k = 0; k < kNaScanItems; ++k) {
    const int64_t i = base + k;
    const int64_t x = i < nrow ? v.counts[i] : 0;
    vals[k] = run;
    run += x;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t incl = run;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const int64_t w = lane < kNaScanBlock / 32 ? warp_tot[lane] : 0;
    int64_t wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kNaScanBlock / 32) warp_tot[lane] = wi - w;
  }
  __syncthreads();
  const int64_t excl = incl - run + warp_tot[wid] + v.tile_off[blockIdx.x];
  for (int k = 0; k < kNaScanItems; ++k) {
    const int64_t i = base + k;
    if (i < nrow) v.offsets[i] = vals[k] + excl;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) v.offsets[nrow] = v.tile_off[ntiles];
}

__global__ void na_bucket_k(View v, const int64_t* __restrict__ rows, int64_t n, int64_t nrow) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = rows[s] - 1;
    if (r < 0 || r >= nrow) continue;
    const int32_t pos = atomicAdd(&v.cursor[r], 1);
    v.order[v.offsets[r] + pos] = (uint32_t)s;
  }
}

// One warp per row: sort the row's entry indices ascending (bitonic network
// in its "flip" form, valid for any length), then add the values in order.
constexpr int kNaSortCap = 256;

__global__ void __launch_bounds__(256) na_sum_k(View v, const double* __restrict__ vals, int64_t nrow,
                                                double* __restrict__ out) {
  __shared__ uint32_t sh[256 / 32][kNaSortCap];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // a row number out of range (flagged by na_count_k, earlier on the stream)
  // fails the call: out keeps its contents, as with the allocating path
  if (*(volatile int*)v.bad) return;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x / 32) + wid; r < nrow; r += warps) {
    const int64_t b = v.offsets[r];
    const int64_t n = v.offsets[r + 1] - b;
    uint32_t* a = v.order + b;
    if (n <= kNaSortCap) {
      for (int64_t t = lane; t < n; t += 32) sh[wid][t] = a[t];
      __syncwarp();
      a = sh[wid];
    }
    if (n > 1) {
      int64_t npow = 1;
      while (npow < n) npow <<= 1;
      const int64_t half = npow >> 1;
      for (int64_t size = 2; size <= npow; size <<= 1) {
        const int64_t h = size >> 1;
        for (int64_t p = lane; p < half; p += 32) {
          const int64_t blk = p / h, off = p - blk * h;
          const int64_t i = blk * size + off, j = blk * size + size - 1 - off;
          if (j < n && a[i] > a[j]) { const uint32_t x = a[i]; a[i] = a[j]; a[j] = x; }
        }
        __syncwarp();
        for (int64_t stride = h >> 1; stride > 0; stride >>= 1) {
          for (int64_t p = lane; p < half; p += 32) {
            const int64_t blk = p / stride, off = p - blk * stride;
            const int64_t i = blk * 2 * stride + off, j = i + stride;
            if (j < n && a[i] > a[j]) { const uint32_t x = a[i]; a[i] = a[j]; a[j] = x; }
          }
          __syncwarp();
        }
      }
    }
    if (lane == 0) {
      // from +0, as the allocating path and SysvecAssembler (which adds into
      // zeros(T, n)): a row of negative zeros sums to +0
      double s = 0.0;
      for (int64_t t = 0; t < n; ++t) s = __dadd_rn(s, vals[a[t]]);
      out[r] = s;
    }
    __syncwarp();
  }
}

}  // namespace

using namespace elfel;

extern "C" int elfel_sysvec_assemble_noalloc(elfel_ctx* h, int64_t nrow, const int64_t* d_rows, const double* d_vals,
                                             int64_t n, double* d_out) {
  if (!h) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  if (nrow < 0 || n < 0) return fail(c, ELFEL_ERR_ARG, "sysvec_noalloc: negative size");
  if (nrow > kNaMaxRows || n > kNaMaxEntries)
    return fail(c, ELFEL_ERR_ARG,
                "sysvec_noalloc: %lld rows / %lld entries exceed the fixed scratch (at most %lld rows and %lld "
                "entries); use elfel_sysvec_assemble",
                (long long)nrow, (long long)n, (long long)kNaMaxRows, (long long)kNaMaxEntries);
  if ((n > 0 && (!d_rows || !d_vals)) || (nrow > 0 && !d_out)) return fail(c, ELFEL_ERR_ARG, "sysvec_noalloc: NULL");
  if (c->device < 0 || c->device >= kMaxDevices) return fail(c, ELFEL_ERR_ARG, "sysvec_noalloc: device index");
  ELFEL_CUDA(c, cudaSetDevice(c->device));
  void* base = nullptr;
  {
    // first call on this device: resolve the device address of the scratch
    // array (with the device current); later calls reuse it
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[c->device]) {
      void* p = nullptr;
      ELFEL_CUDA(c, cudaGetSymbolAddress(&p, g_na_scratch));
      g_na_addr[c->device] = p;
    }
    base = g_na_addr[c->device];
  }
  if (nrow == 0) {
    if (n > 0) return fail(c, ELFEL_ERR_ARG, "sysvec_noalloc: %lld entries but no rows (every row out of range)",
                           (long long)n);
    return ELFEL_OK;
  }
  const View v = carve(base);
  cudaStream_t st = c->stream;
  const unsigned g1 = grid_for(nrow, 256, (int64_t)c->sm_count * 8);
  na_clear_k<<<g1, 256, 0, st>>>(v, nrow);
  if (n > 0) na_count_k<<<grid_for(n, 256, (int64_t)c->sm_count * 8), 256, 0, st>>>(v, d_rows, n, nrow);
  const int64_t ntiles = (nrow + kNaTile - 1) / kNaTile;
  na_tile_tot_k<<<(unsigned)ntiles, kNaScanBlock, 0, st>>>(v, nrow);
  na_tile_scan_k<<<1, 1, 0, st>>>(v, ntiles);
  na_tile_k<<<(unsigned)ntiles, kNaScanBlock, 0, st>>>(v, nrow, ntiles);
  if (n > 0) na_bucket_k<<<grid_for(n, 256, (int64_t)c->sm_count * 8), 256, 0, st>>>(v, d_rows, n, nrow);
  na_sum_k<<<grid_for(nrow, 8, (int64_t)c->sm_count * 16), 256, 0, st>>>(v, d_vals, nrow, d_out);
  ELFEL_LAUNCH_CHECK(c);
  int hbad = 0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&hbad, v.bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  ELFEL_CUDA(c, cudaStreamSynchronize(st));
  if (hbad) return fail(c, ELFEL_ERR_ARG, "sysvec_noalloc: row number outside 1..%lld", (long long)nrow);
  return ELFEL_OK;
}
