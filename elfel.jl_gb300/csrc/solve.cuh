// Device solvers for K[1:nu,1:nu] x = F[1:nu] - (K*T)[1:nu]: the per-system
// solver data shared by the one-system drivers (solve.cu) and the batched
// engine (batch.cu), and the SELL-C-sigma row kernel both use.
#pragma once
#include "sysmat.cuh"

namespace elfel {

constexpr int kBlk = 256;
constexpr int kGraphIters = 16;
constexpr int kMaxRedBlocks = 2048;  // partial-sum slots per reduction area
constexpr int kVecOcc = 8;           // register budget of vector kernels: 8 blocks/SM (32 registers)
constexpr int kGridCap = 152 * kVecOcc;
constexpr int kVecGridCap = 152 * kVecOcc;  // vector kernels: one full wave (4 blocks/SM measured slower)
constexpr int kSellOcc = 4;           // FP64 SELL kernels: <= 64 registers, 4 blocks/SM
// FP32 SELL kernels fit their 8-deep unroll in 40 registers: 6 blocks/SM.
template <typename T>
constexpr int sell_occ() { return sizeof(T) == 4 ? 6 : kSellOcc; }
constexpr int kSigma = 256;          // row-sorting window

// device scalar slots
enum {
  S_PQ = 0, S_RZ, S_RR, S_BETA, S_BN2, S_TOL2, S_RMAX, S_DELTA,
  S_ALPHA,  // rz / pq, computed once by the SpMV's last block
  S_SCALE,  // FP32 refinement: the FP32 residual is (FP64 residual) / S_SCALE
  S_BN2S,   // ||b||^2 / S_SCALE^2: the FP32 recurrence's convergence threshold
  // MINRES
  S_GAM, S_GAMP, S_GAMN, S_DEL, S_C, S_CP, S_S, S_SP, S_ETA, S_ETA0, S_A1, S_A2, S_A3, S_CN,
  S_COUNT
};
// device int flags
enum { F_DONE = 0, F_RU, F_ITER, F_MAXIT, F_ROT, F_CONV, F_BRK, F_COUNT };

struct Red4 {
  double* partials;  // kMaxRedBlocks x 4
  unsigned* ticket;
};

// CSR in the original order (rows 0..nu-1): free part (col < nu) and data part.
struct Csr {
  int64_t nrows = 0, nnz = 0;
  DBuf<int32_t> rowptr, col, map;  // map: index into the CSC values
  DBuf<double> v64;
  void release(Ctx* c) {
    rowptr.release(c); col.release(c); map.release(c); v64.release(c);
    nrows = nnz = 0;
  }
};

// SELL-C-sigma matrix of the free-free block (permuted rows and columns).
struct Sell {
  int64_t nrows = 0, nslices = 0, nnz_pad = 0;
  int d16 = 0;
  DBuf<int64_t> sptr;   // nslices + 1 entry offsets
  DBuf<int32_t> sw;     // slice widths
  DBuf<int16_t> dcol;   // d16: column - row (permuted)
  DBuf<int32_t> col;    // !d16: column (permuted)
  DBuf<int32_t> map;    // CSC index of each entry, -1 for padding
  DBuf<int32_t> perm;   // permuted row -> original row
  DBuf<double> v64;
  DBuf<float> v32;
  void release(Ctx* c) {
    sptr.release(c); sw.release(c); dcol.release(c); col.release(c); map.release(c); perm.release(c);
    v64.release(c); v32.release(c);
    nrows = nslices = nnz_pad = 0;
  }
};

// POD view passed to kernels.
struct SellView {
  int64_t nrows, nslices;
  const int64_t* sptr;
  const int32_t* sw;
  const int16_t* d16;
  const int32_t* c32;
};

struct SolverData {
  int64_t nu = -1;
  const void* pattern_id = nullptr;
  int64_t pattern_nnz = -1;
  int group = 4;  // lanes per row of the CSR kernels (lifting, final residual)
  Csr ff, fd;
  Sell A;
  // original order
  DBuf<double> T64, bo64, xo64, ro64, dinvo;
  // permuted order
  DBuf<double> dinv64, b64, x64, r64, z64, p64, q64, y64;
  DBuf<float> dinv32, r32, p32, q32, z32, xa32, zz32, b32, x32;
  DBuf<double> v64[3], w64[3];
  DBuf<float> v32[3], w32[3];
  DBuf<double> scal;
  DBuf<int> flags;
  DBuf<double> red;  // 3 reduction areas
  DBuf<unsigned> tickets;
  cudaGraphExec_t g_pcg64 = nullptr, g_pcg32 = nullptr, g_minres64 = nullptr, g_minres32 = nullptr;
  SellView view() const {
    return SellView{A.nrows, A.nslices, A.sptr.p, A.sw.p, A.d16 ? A.dcol.p : nullptr, A.d16 ? nullptr : A.col.p};
  }
  void release(Ctx* c) {
    ff.release(c); fd.release(c); A.release(c);
    for (DBuf<double>* b : {&T64, &bo64, &xo64, &ro64, &dinvo, &dinv64, &b64, &x64, &r64, &z64, &p64, &q64, &y64})
      b->release(c);
    for (DBuf<float>* b : {&dinv32, &r32, &p32, &q32, &z32, &xa32, &zz32, &b32, &x32}) b->release(c);
    for (int i = 0; i < 3; ++i) { v64[i].release(c); w64[i].release(c); v32[i].release(c); w32[i].release(c); }
    scal.release(c); flags.release(c); red.release(c); tickets.release(c);
    for (cudaGraphExec_t* g : {&g_pcg64, &g_pcg32, &g_minres64, &g_minres32})
      if (*g) { cudaGraphExecDestroy(*g); *g = nullptr; }
  }
};

void solver_release(Ctx* c, elfel_sysmat* m);

// Solver structures (CSR split, SELL-C-sigma) of the leading nu x nu block;
// kept while the pattern and nu stay the same.
int build_solver(elfel_sysmat* m, int64_t nu);
// Solver values from the CSC values.  abs_diag: |K_ii| preconditioner
// (MINRES); diff32: the FP32 copy in difference form (FP32 CG).
int refresh_values(elfel_sysmat* m, int abs_diag, int diff32);
// Lifted right-hand side b = F[1:nu] - (K*T)[1:nu] of solve!: T (n values)
// is copied from the host (t_dev = 0) or the device; F from the host, or the
// assembled rhs when F is null.  Leaves b in the permuted order in S->b64, the
// original order in S->bo64 and ||b||^2 in scal[S_BN2] (device; no host sync).
int lift_rhs(elfel_sysmat* m, const double* F, const double* T, int t_dev);
// x64 (permuted order) back to the original order in S->xo64 and the FP64
// residual of the original system there; rr = ||b - K_ff x||^2 in scal[S_RR]
// (device).
int solution_residual(elfel_sysmat* m);

// ------------------------------------------------------------------ launches
// Programmatic dependent launch: the iteration kernels of the captured graphs
// are launched with programmatic stream serialization, so the next kernel is
// scheduled while this one runs; it waits (griddepcontrol.wait) until this
// grid has completed and its writes are visible before touching its data.
// Without the launch attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Off by default: measured on GB300 it gained nothing over plain graph
// launches and slowed the FP64 one-system iteration at mid sizes; ELFEL_PDL=1
// in the environment switches it on (for comparison).
inline bool pdl_enabled() {
  static const bool on = [] {
    const char* e = getenv("ELFEL_PDL");
    return e && e[0] == '1';
  }();
  return on;
}

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*k)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// ------------------------------------------------------------------ SELL rows
template <bool D16>
__device__ __forceinline__ int sell_col(const SellView& A, int64_t k, int64_t row) {
  if (D16) return (int)row + (int)__ldcs(A.d16 + k);
  return __ldcs(A.c32 + k);
}

// The x term of one stored entry.  Plain form: x_c.  Difference form (DIFF):
// the matrix is stored with its row sums s_i in the diagonal slots, and
//   y_i = s_i x_i + sum_{j != i} a_ij (x_j - x_i),
// an identity for any matrix; for slowly varying x the differences are exact
// (Sterbenz), so in FP32 the near-zero row sums of stiffness matrices do not
// cancel catastrophically and the smallest eigenvalues are kept.  Padding
// entries have value 0 and column = row, so they add nothing either way.
template <typename T, bool DIFF>
__device__ __forceinline__ T xterm(const T xc, int c, int64_t row, T xi) {
  if (!DIFF) return xc;
  return (int64_t)c == row ? xi : xc - xi;
}

// A gathered entry of x: through the read-only path when x does not change
// during the kernel, else (COH: a persistent kernel in which other blocks
// write x between its phases) through L2.
template <typename T, bool COH>
__device__ __forceinline__ T xload(const T* p) {
  return COH ? __ldcg(p) : __ldg(p);
}

// (A x)_row for row = s * 32 + lane of slice s (0 for lanes past the last
// row); xi = x[row] in the difference form.  Eight entries per lane in
// flight: all column and value loads of a group are issued before the
// dependent gathers of x.
template <typename T, bool D16, bool DIFF, bool COH = false>
__device__ __forceinline__ T sell_row_acc(const SellView& A, const T* __restrict__ v, const T* x,
                                          int64_t s, int lane, T xi) {
  const int64_t base = A.sptr[s] + lane;
  const int64_t row = s * 32 + lane;
  const int w = row < A.nrows ? A.sw[s] : 0;  // lanes past the last row stay idle
  T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  int j = 0;
  for (; j + 7 < w; j += 8) {
    const int64_t k = base + (int64_t)j * 32;
    int cc[8];
    T vv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) cc[u] = sell_col<D16>(A, k + 32 * u, row);
#pragma unroll
    for (int u = 0; u < 8; ++u) vv[u] = __ldcs(v + k + 32 * u);
    T xx[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) xx[u] = xterm<T, DIFF>(xload<T, COH>(x + cc[u]), cc[u], row, xi);
    a0 += vv[0] * xx[0];
    a1 += vv[1] * xx[1];
    a2 += vv[2] * xx[2];
    a3 += vv[3] * xx[3];
    a0 += vv[4] * xx[4];
    a1 += vv[5] * xx[5];
    a2 += vv[6] * xx[6];
    a3 += vv[7] * xx[7];
  }
  if (j + 3 < w) {
    const int64_t k = base + (int64_t)j * 32;
    const int c0 = sell_col<D16>(A, k, row), c1 = sell_col<D16>(A, k + 32, row);
    const int c2 = sell_col<D16>(A, k + 64, row), c3 = sell_col<D16>(A, k + 96, row);
    const T v0 = __ldcs(v + k), v1 = __ldcs(v + k + 32), v2 = __ldcs(v + k + 64), v3 = __ldcs(v + k + 96);
    a0 += v0 * xterm<T, DIFF>(xload<T, COH>(x + c0), c0, row, xi);
    a1 += v1 * xterm<T, DIFF>(xload<T, COH>(x + c1), c1, row, xi);
    a2 += v2 * xterm<T, DIFF>(xload<T, COH>(x + c2), c2, row, xi);
    a3 += v3 * xterm<T, DIFF>(xload<T, COH>(x + c3), c3, row, xi);
    j += 4;
  }
  for (; j < w; ++j) {
    const int64_t k = base + (int64_t)j * 32;
    const int cj = sell_col<D16>(A, k, row);
    a0 += __ldcs(v + k) * xterm<T, DIFF>(xload<T, COH>(x + cj), cj, row, xi);
  }
  return (a0 + a1) + (a2 + a3);
}

// (A x)_row in FP64 for row = s * 32 + lane, one entry at a time (residuals).
template <bool D16, bool COH = false>
__device__ __forceinline__ double sell_row_resid(const SellView& A, const double* __restrict__ v, const double* x,
                                                 int64_t s, int lane) {
  const int64_t base = A.sptr[s] + lane;
  const int64_t row = s * 32 + lane;
  const int w = row < A.nrows ? A.sw[s] : 0;
  double acc = 0.0;
  for (int j = 0; j < w; ++j) {
    const int64_t k = base + (int64_t)j * 32;
    acc += __ldcs(v + k) * xload<double, COH>(x + sell_col<D16>(A, k, row));
  }
  return acc;
}

}  // namespace elfel
