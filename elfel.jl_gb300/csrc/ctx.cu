// Context, device memory accounting, errors and the device scan.
#include <stdarg.h>
#include <stdlib.h>

#include "common.cuh"

namespace elfel {

int fail(Ctx* c, int code, const char* fmt, ...) {
  if (c) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->last_error = buf;
  }
  return code;
}

int dalloc(Ctx* c, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return ELFEL_OK;
  if (c->budget > 0 && c->in_use + (int64_t)bytes > c->budget)
    return fail(c, ELFEL_ERR_BUDGET, "device memory budget exceeded: in use %lld + request %zu > budget %lld",
                (long long)c->in_use, bytes, (long long)c->budget);
  cudaError_t e = c->pool ? cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream) : cudaMallocAsync(p, bytes, c->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, ELFEL_ERR_BUDGET, "device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
  }
  c->in_use += (int64_t)bytes;
  if (c->in_use > c->peak) c->peak = c->in_use;
  return ELFEL_OK;
}

void dfree(Ctx* c, void* p, size_t bytes) {
  if (!p) return;
  cudaFreeAsync(p, c->stream);
  c->in_use -= (int64_t)bytes;
}

int red_scratch(Ctx* c, int nslots, int nblocks, RedSlot* slots) {
  size_t per = (size_t)nblocks * sizeof(double) + 256;
  size_t need = per * (size_t)nslots;
  if (need > c->red_scratch_bytes) {
    if (c->red_scratch) dfree(c, c->red_scratch, c->red_scratch_bytes);
    c->red_scratch = nullptr;
    c->red_scratch_bytes = 0;
    ELFEL_TRY(dalloc(c, &c->red_scratch, need));
    c->red_scratch_bytes = need;
    ELFEL_CUDA(c, cudaMemsetAsync(c->red_scratch, 0, need, c->stream));
  }
  char* base = (char*)c->red_scratch;
  for (int s = 0; s < nslots; ++s) {
    slots[s].partials = (double*)(base + per * s);
    slots[s].ticket = (unsigned int*)(base + per * s + (size_t)nblocks * sizeof(double));
  }
  return ELFEL_OK;
}

// ------------------------------------------------------------------ scan
// Three-phase exclusive scan: per-block totals, recursive scan of the totals,
// then a block-local scan with the block offset added.
constexpr int kScanBlock = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

template <typename TIn>
__global__ void scan_block_totals_k(const TIn* in, int64_t n, int64_t* totals) {
  __shared__ int64_t sh[kScanBlock / 32];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + (int64_t)k * kScanBlock + threadIdx.x;
    if (i < n) s += (int64_t)in[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < kScanBlock / 32; ++w) t += sh[w];
    totals[blockIdx.x] = t;
  }
}

// Block-local exclusive scan of a tile; each thread owns kScanItems
// consecutive items.  offsets = exclusive scan of the block totals.
template <typename TIn>
__global__ void scan_tile_k(const TIn* in, int64_t n, const int64_t* offsets, int64_t* out) {
  __shared__ int64_t warp_tot[kScanBlock / 32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t run = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    int64_t x = i < n ? (int64_t)in[i] : 0;
    v[k] = run;
    run += x;
  }
  // exclusive scan of the per-thread totals across the block
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int64_t w = lane < kScanBlock / 32 ? warp_tot[lane] : 0;
    int64_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanBlock / 32) warp_tot[lane] = wi - w;
  }
  __syncthreads();
  int64_t excl = incl - run + warp_tot[wid] + offsets[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    if (i < n) out[i] = v[k] + excl;
  }
}

__global__ void write_total_k(const int64_t* offsets, int64_t nblocks, const int64_t* totals, int64_t* out_total) {
  *out_total = offsets[nblocks - 1] + totals[nblocks - 1];
}

template <typename TIn>
static int scan_impl(Ctx* c, const TIn* in, int64_t n, int64_t* out) {
  if (n <= 0) {
    ELFEL_CUDA(c, cudaMemsetAsync(out, 0, sizeof(int64_t), c->stream));
    return ELFEL_OK;
  }
  int64_t nb = (n + kScanTile - 1) / kScanTile;
  DBuf<int64_t> totals, offsets;
  ELFEL_TRY(totals.alloc(c, (size_t)nb));
  ELFEL_TRY(offsets.alloc(c, (size_t)nb + 1));
  scan_block_totals_k<TIn><<<(unsigned)nb, kScanBlock, 0, c->stream>>>(in, n, totals.p);
  ELFEL_LAUNCH_CHECK(c);
  if (nb == 1) {
    ELFEL_CUDA(c, cudaMemsetAsync(offsets.p, 0, sizeof(int64_t), c->stream));
  } else {
    ELFEL_TRY(scan_impl<int64_t>(c, totals.p, nb, offsets.p));
  }
  scan_tile_k<TIn><<<(unsigned)nb, kScanBlock, 0, c->stream>>>(in, n, offsets.p, out);
  ELFEL_LAUNCH_CHECK(c);
  write_total_k<<<1, 1, 0, c->stream>>>(offsets.p, nb, totals.p, out + n);
  ELFEL_LAUNCH_CHECK(c);
  totals.release(c);
  offsets.release(c);
  return ELFEL_OK;
}

int exclusive_scan_i64(Ctx* c, int64_t* data, int64_t n) {
  // in-place: scan_tile reads its own items before writing them, and reads
  // only its own tile, so in == out is safe.
  return scan_impl<int64_t>(c, data, n, data);
}

int scan_counts_i32(Ctx* c, const int32_t* counts, int64_t n, int64_t* offsets) {
  return scan_impl<int32_t>(c, counts, n, offsets);
}

}  // namespace elfel

// ------------------------------------------------------------------ C ABI
using namespace elfel;

static void clear_phases(Ctx* c);

extern "C" int elfel_abi_version(void) { return ELFEL_ABI_VERSION; }

extern "C" int elfel_ctx_create(int device, int64_t mem_budget_bytes, elfel_ctx** out) {
  if (!out) return ELFEL_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return ELFEL_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return ELFEL_ERR_CUDA;
  elfel_ctx* h = new elfel_ctx();
  h->c.device = device;
  h->c.budget = mem_budget_bytes;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) h->c.sm_count = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&h->c.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return ELFEL_ERR_CUDA;
  }
  h->c.own_stream = h->c.stream;
  // A pool of the context's own: memory freed by one assembly (the pattern
  // builder's sort keys, a replaced system's buffers) stays mapped for the
  // next one instead of going back to the driver at every synchronisation.
  // It keeps up to the memory budget (everything without one).
  {
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&h->c.pool, &props) == cudaSuccess) {
      uint64_t keep = mem_budget_bytes > 0 ? (uint64_t)mem_budget_bytes : UINT64_MAX;
      cudaMemPoolSetAttribute(h->c.pool, cudaMemPoolAttrReleaseThreshold, &keep);
    } else {
      cudaGetLastError();
      h->c.pool = nullptr;  // the device's default pool then
    }
  }
  {
    // Kernels read pageable host memory in place only where the device walks
    // the host's page tables (ATS, as on Grace); with HMM alone an access
    // faults and migrates pages, and the copy engines are used instead.
    int pa = 0, hpt = 0;
    if (cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess) {
      cudaGetLastError();
      pa = hpt = 0;
    }
    h->c.pageable_access = pa && hpt;
  }
  const char* tr = getenv("ELFEL_TRACE");
  h->c.trace = (tr && tr[0] == '1') ? 1 : 0;
  const char* tu = getenv("ELFEL_TUNE");
  h->c.tune = (tu && tu[0] == '0') ? 0 : 1;
  const char* ti = getenv("ELFEL_TILES");
  h->c.tiles = (ti && ti[0] == '0') ? 0 : 1;
  *out = h;
  return ELFEL_OK;
}

namespace elfel {

int aux_fork(Ctx* c, cudaStream_t* aux) {
  if (!c->aux) {
    ELFEL_CUDA(c, cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    ELFEL_CUDA(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    ELFEL_CUDA(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
  }
  ELFEL_CUDA(c, cudaEventRecord(c->ev_fork, c->stream));
  ELFEL_CUDA(c, cudaStreamWaitEvent(c->aux, c->ev_fork, 0));
  *aux = c->aux;
  return ELFEL_OK;
}

int aux_after(Ctx* c, cudaEvent_t ev, cudaStream_t* aux) {
  if (!c->aux) {
    ELFEL_CUDA(c, cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    ELFEL_CUDA(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    ELFEL_CUDA(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
  }
  ELFEL_CUDA(c, cudaStreamWaitEvent(c->aux, ev, 0));
  *aux = c->aux;
  return ELFEL_OK;
}

int aux_join(Ctx* c) {
  if (!c->aux) return ELFEL_OK;
  ELFEL_CUDA(c, cudaEventRecord(c->ev_join, c->aux));
  ELFEL_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_join, 0));
  return ELFEL_OK;
}

const void* host_device_ptr(Ctx* c, const void* host, int* pinned) {
  if (pinned) *pinned = 0;
  if (!host) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return host;
  if (a.type == cudaMemoryTypeHost) {
    if (pinned) *pinned = a.devicePointer != nullptr;
    return a.devicePointer;
  }
  return c->pageable_access ? host : nullptr;
}

void tune_record(Ctx* c, const char* key, const std::string& cand, int best, const std::vector<double>& ms) {
  std::string line = std::string(key) + ":";
  size_t pos = 0;
  for (size_t k = 0; k < ms.size(); ++k) {
    const size_t e = cand.find(',', pos);
    const std::string name = cand.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
    pos = e == std::string::npos ? cand.size() : e + 1;
    char one[96];
    snprintf(one, sizeof(one), " %s=%.4fms", name.c_str(), ms[k]);
    line += one;
    if ((int)k == best) line += "*";
  }
  for (size_t i = 0; i < c->tune_keys.size(); ++i)
    if (c->tune_keys[i] == key) {
      c->tune_lines[i] = line;
      c->tune_choice[i] = best;
      return;
    }
  c->tune_keys.push_back(key);
  c->tune_lines.push_back(line);
  c->tune_choice.push_back(best);
}

int tune_lookup(const Ctx* c, const char* key) {
  for (size_t i = 0; i < c->tune_keys.size(); ++i)
    if (c->tune_keys[i] == key) return c->tune_choice[i];
  return -1;
}

}  // namespace elfel

// FMA throughput probe: 8 independent FMA chains per thread, one full wave.
template <typename T>
__global__ void __launch_bounds__(256) fma_rate_k(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == (T)-1) out[0] = s;  // never true for these inputs; keeps the chains live
}

extern "C" int elfel_ctx_fma_rate(elfel_ctx* h, int32_t bits, double* tflops) {
  if (!h || !tflops || (bits != 32 && bits != 64)) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  cudaSetDevice(c->device);
  DBuf<double> out;
  ELFEL_TRY(out.alloc(c, 1));
  const unsigned grid = (unsigned)c->sm_count * 8;
  const int iters = bits == 64 ? 1 << 12 : 1 << 15;
  cudaEvent_t e0, e1;
  ELFEL_CUDA(c, cudaEventCreate(&e0));
  ELFEL_CUDA(c, cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {  // the first run warms up
    ELFEL_CUDA(c, cudaEventRecord(e0, c->stream));
    if (bits == 64) fma_rate_k<double><<<grid, 256, 0, c->stream>>>(out.p, iters, 0.999999, 1e-7);
    else fma_rate_k<float><<<grid, 256, 0, c->stream>>>((float*)out.p, iters, 0.999999f, 1e-7f);
    ELFEL_CUDA(c, cudaEventRecord(e1, c->stream));
    ELFEL_CUDA(c, cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  out.release(c);
  *tflops = 2.0 * 8.0 * iters * (double)grid * 256.0 / (best * 1e-3) / 1e12;
  return ELFEL_OK;
}

extern "C" int elfel_ctx_tuning(const elfel_ctx* h, int index, char* line, int cap, int32_t* choice) {
  if (!h) return ELFEL_ERR_ARG;
  const Ctx* c = &h->c;
  if (index < 0 || index >= (int)c->tune_lines.size()) return ELFEL_ERR_ARG;
  if (line && cap > 0) snprintf(line, (size_t)cap, "%s", c->tune_lines[index].c_str());
  if (choice) *choice = c->tune_choice[index];
  return ELFEL_OK;
}

extern "C" int elfel_ctx_destroy(elfel_ctx* h) {
  if (!h) return ELFEL_OK;
  cudaSetDevice(h->c.device);
  if (h->c.red_scratch) dfree(&h->c, h->c.red_scratch, h->c.red_scratch_bytes);
  cudaStreamSynchronize(h->c.stream);
  clear_phases(&h->c);
  if (h->c.own_stream) cudaStreamDestroy(h->c.own_stream);
  if (h->c.aux) {
    cudaStreamSynchronize(h->c.aux);
    cudaStreamDestroy(h->c.aux);
  }
  if (h->c.ev_fork) cudaEventDestroy(h->c.ev_fork);
  if (h->c.ev_join) cudaEventDestroy(h->c.ev_join);
  // memory still held by live systems is released once they free it
  if (h->c.pool) cudaMemPoolDestroy(h->c.pool);
  delete h;
  return ELFEL_OK;
}

extern "C" const char* elfel_ctx_last_error(const elfel_ctx* h) {
  return h ? h->c.last_error.c_str() : "null context";
}

extern "C" int elfel_ctx_memory(const elfel_ctx* h, int64_t* in_use, int64_t* peak) {
  if (!h) return ELFEL_ERR_ARG;
  if (in_use) *in_use = h->c.in_use;
  if (peak) *peak = h->c.peak;
  return ELFEL_OK;
}

extern "C" int elfel_ctx_set_stream(elfel_ctx* h, void* s) {
  if (!h) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stream = s ? (cudaStream_t)s : c->own_stream;
  return ELFEL_OK;
}

extern "C" void* elfel_ctx_stream(const elfel_ctx* h) { return h ? (void*)h->c.stream : nullptr; }

static void clear_phases(Ctx* c) {
  for (PhaseRec& r : c->phases) {
    if (r.start) cudaEventDestroy(r.start);
    if (r.stop) cudaEventDestroy(r.stop);
  }
  c->phases.clear();
}

extern "C" int elfel_ctx_profile(elfel_ctx* h, int enable) {
  if (!h) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  cudaSetDevice(c->device);
  if (enable) {
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    clear_phases(c);
  }
  c->profiling = enable ? 1 : 0;
  return ELFEL_OK;
}

extern "C" int elfel_ctx_profile_read(elfel_ctx* h, int index, char* name, int name_cap, double* total_ms,
                                      int64_t* count) {
  if (!h) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  cudaSetDevice(c->device);
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  // distinct names in first-seen order
  std::vector<std::string> names;
  for (const PhaseRec& r : c->phases) {
    bool seen = false;
    for (const std::string& n : names) seen = seen || n == r.name;
    if (!seen) names.push_back(r.name);
  }
  if (index < 0 || index >= (int)names.size()) return ELFEL_ERR_ARG;
  double ms = 0.0;
  int64_t k = 0;
  for (const PhaseRec& r : c->phases) {
    if (r.name != names[index]) continue;
    float t = 0.0f;
    ELFEL_CUDA(c, cudaEventElapsedTime(&t, r.start, r.stop));
    ms += t;
    ++k;
  }
  if (name && name_cap > 0) {
    snprintf(name, (size_t)name_cap, "%s", names[index].c_str());
  }
  if (total_ms) *total_ms = ms;
  if (count) *count = k;
  return ELFEL_OK;
}

extern "C" int elfel_ctx_synchronize(elfel_ctx* h) {
  if (!h) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  return ELFEL_OK;
}
