// Shared definitions of the GB300 element-assembly / sparse-solve library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/elfel_gpu.h"

namespace elfel {

constexpr int kWarp = 32;
constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs; grids are sized in multiples of this

// ------------------------------------------------------------------ context
struct PhaseRec {
  std::string name;
  cudaEvent_t start = nullptr, stop = nullptr;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;      // stream all work is issued on
  cudaStream_t own_stream = nullptr;  // the context's own stream
  cudaStream_t aux = nullptr;         // second stream for uploads that overlap work on `stream` (lazy)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int pageable_access = 0;            // kernels may read pageable host memory in place (ATS)
  cudaMemPool_t pool = nullptr;  // the context's stream-ordered pool (keeps freed memory for reuse)
  int64_t budget = 0;       // bytes the context may hold on the device (0 = unlimited)
  int64_t in_use = 0;       // bytes currently held
  int64_t peak = 0;
  int sm_count = kSMs;
  int trace = 0;  // ELFEL_TRACE=1: solver progress on stderr
  std::string last_error;
  // scratch for deterministic reductions (partials + counters), grown on demand
  void* red_scratch = nullptr;
  size_t red_scratch_bytes = 0;
  // phase timing: CUDA events recorded on `stream` around each kernel launch
  int profiling = 0;
  std::vector<PhaseRec> phases;
  // tile reduction of resident T6 heat patterns: on unless ELFEL_TILES=0
  int tiles = 1;
  // autotuner: on unless ELFEL_TUNE=0; one line per tuned key
  int tune = 1;
  std::vector<std::string> tune_lines;
  std::vector<std::string> tune_keys;
  std::vector<int> tune_choice;
};

// Record the autotuner's timings of the candidates (names comma-separated in
// cand) for key and the chosen index; replaces an earlier record of the key.
void tune_record(Ctx* c, const char* key, const std::string& cand, int best, const std::vector<double>& ms);
// The recorded choice for key, or -1.
int tune_lookup(const Ctx* c, const char* key);

// Records a start event on construction and a stop event on destruction when
// the context is profiling; otherwise does nothing.
struct Phase {
  Ctx* c;
  int idx = -1;
  Phase(Ctx* ctx, const char* name) : c(ctx) {
    if (!c->profiling) return;
    PhaseRec r;
    r.name = name;
    if (cudaEventCreate(&r.start) != cudaSuccess || cudaEventCreate(&r.stop) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    cudaEventRecord(r.start, c->stream);
    c->phases.push_back(r);
    idx = (int)c->phases.size() - 1;
  }
  ~Phase() {
    if (idx >= 0) cudaEventRecord(c->phases[idx].stop, c->stream);
  }
};

// Record an error message on the context and return the code.
int fail(Ctx* c, int code, const char* fmt, ...);

// Check a CUDA call; on failure record and return ELFEL_ERR_CUDA from the caller.
#define ELFEL_CUDA(ctx, call)                                                         \
  do {                                                                                \
    cudaError_t _e = (call);                                                          \
    if (_e != cudaSuccess)                                                            \
      return ::elfel::fail((ctx), ELFEL_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, \
                           #call, cudaGetErrorString(_e));                            \
  } while (0)

#define ELFEL_TRY(expr)       \
  do {                        \
    int _rc = (expr);         \
    if (_rc != ELFEL_OK) return _rc; \
  } while (0)

#define ELFEL_LAUNCH_CHECK(ctx) ELFEL_CUDA(ctx, cudaGetLastError())

// The context's auxiliary stream, made to wait for the work issued on
// c->stream so far (fork); join() makes c->stream wait for it.
int aux_fork(Ctx* c, cudaStream_t* aux);
int aux_join(Ctx* c);
// The auxiliary stream, made to wait only for the event ev (recorded on
// c->stream earlier); join with aux_join.
int aux_after(Ctx* c, cudaEvent_t ev, cudaStream_t* aux);

// A device-usable address of a host array: the device address of pinned
// memory, the host address itself where kernels read pageable memory (ATS),
// else nullptr (the caller then copies with cudaMemcpyAsync).
// *pinned (optional) = 1 for page-locked memory (copy engines work
// asynchronously on it).
const void* host_device_ptr(Ctx* c, const void* host, int* pinned = nullptr);

// Device allocation accounted against the context budget (stream-ordered).
int dalloc(Ctx* c, void** p, size_t bytes);
void dfree(Ctx* c, void* p, size_t bytes);

// A typed device buffer owned by a context.
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  int alloc(Ctx* c, size_t count) {
    release(c);
    if (count == 0) return ELFEL_OK;
    void* q = nullptr;
    int rc = dalloc(c, &q, count * sizeof(T));
    if (rc != ELFEL_OK) return rc;
    p = static_cast<T*>(q);
    n = count;
    return ELFEL_OK;
  }
  // Grow (discarding contents) when the requested count exceeds the capacity.
  int ensure(Ctx* c, size_t count) {
    if (count <= n && p) return ELFEL_OK;
    return alloc(c, count);
  }
  void release(Ctx* c) {
    if (p) dfree(c, p, n * sizeof(T));
    p = nullptr;
    n = 0;
  }
};

inline unsigned grid_for(int64_t n, int block, int64_t cap = 0) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (cap > 0 && g > cap) g = cap;
  return (unsigned)g;
}

// ------------------------------------------------------------------ scan
// Exclusive prefix sum of n int64 values in place: out[i] = sum_{j<i} in[j],
// writes the total to out[n] (the buffer must hold n+1 entries).
int exclusive_scan_i64(Ctx* c, int64_t* data, int64_t n);
// Exclusive scan of int32 counts into an int64 offsets array (n+1 entries).
int scan_counts_i32(Ctx* c, const int32_t* counts, int64_t n, int64_t* offsets);

// ------------------------------------------------------------------ reductions
// Deterministic block-then-fixed-order sums.  Each block writes a partial,
// the last block to finish (integer ticket) adds the partials in index order.
struct RedSlot {
  double* partials;      // [nblocks]
  unsigned int* ticket;  // one counter, reset by the last block
};
int red_scratch(Ctx* c, int nslots, int nblocks, RedSlot* slots);

constexpr int kRedBlocks = kSMs * 4;  // blocks used by reduction-carrying kernels
constexpr int kRedThreads = 256;

// Sum of a block's per-thread values; result valid in thread 0.
template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < BLOCK / 32; ++w) s += sh[w];
  }
  __syncthreads();
  return s;
}

// Publish a block partial; the last block returns true and writes the total.
__device__ __forceinline__ bool finish_sum(double part, RedSlot r, double* total) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    r.partials[blockIdx.x] = part;
    __threadfence();
    unsigned t = atomicAdd(r.ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double s = 0.0;
    volatile double* pp = r.partials;
    for (unsigned b = 0; b < gridDim.x; ++b) s += pp[b];
    *total = s;
    *r.ticket = 0u;
  }
  return last;
}

}  // namespace elfel

// Opaque handle types of the C ABI.
struct elfel_ctx {
  elfel::Ctx c;
};
