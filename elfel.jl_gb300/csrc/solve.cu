// Device solve of the lifted free-free system of the reference's solve!
// (Elfel.jl test/test_heat.jl:73-76):
//     T[1:nu] = K[1:nu,1:nu] \ (F[1:nu] - (K*T)[1:nu])
// The free DOFs are numbered first (numberdofs!, src/FESpaces.jl:250-259), so
// the free-free block is the leading nu x nu block of K.  The direct solve of
// the reference is replaced by
//   ELFEL_PCG64        Jacobi-preconditioned CG, FP64 throughout;
//   ELFEL_PCG32_IR     Jacobi CG on an FP32 copy of K with FP64 residual
//                      replacement ("reliable updates", Sleijpen & van der
//                      Vorst 1996; used for mixed precision by Clark et al.
//                      2010): the solution is accumulated in FP64, and each
//                      time the FP32 recurrence residual has dropped by a
//                      factor delta the true residual b - K x is recomputed in
//                      FP64 and replaces it; convergence is judged on that
//                      FP64 residual;
//   ELFEL_MINRES64     MINRES (Paige & Saunders 1975) with a symmetric positive
//                      diagonal preconditioner: |K_ii| on rows with a diagonal,
//                      the pressure mass-matrix diagonal on Stokes pressure rows;
//   ELFEL_MINRES32_IR  the same MINRES in FP32 inside FP64 iterative refinement.
//
// Matrix format of the iterations: SELL-C-sigma (Kreutzer et al. 2014) with
// C = 32 rows per slice (one warp, one row per lane) and rows sorted by length
// within windows of sigma = 256 rows, so a slice pads little.  Slices store
// their entries column-major: entry j of the slice's rows is one coalesced
// 32-wide load.  Column indices are 16-bit deltas from the row's own
// (permuted) index when every delta fits, else 32-bit.  The Krylov vectors
// live in the permuted order; the right-hand side goes in and the solution
// comes out through the permutation.  Matrix streams use evict-first loads so
// the gathered vector stays in L2.
//
// All reductions are deterministic (per-block partials added in a fixed
// order).  Iterations run as CUDA graphs of kGraphIters iterations; kernels
// of a finished (or paused) iteration exit at once.
#include <math.h>

#include <chrono>

#include "solve.cuh"

namespace elfel {

void solver_release(Ctx* c, elfel_sysmat* m) {
  if (m->solver) {
    m->solver->release(c);
    delete m->solver;
    m->solver = nullptr;
  }
}

// ------------------------------------------------------------------ reductions
// Sum NV per-thread values over the grid; the last block gets the totals.
// The warp stage adds in the working precision T (FP32 kernels keep the FP64
// pipe free); warp, block and grid totals are then added in FP64.
template <int NV, typename T>
__device__ __forceinline__ bool grid_sums(T (&v)[NV], Red4 red, double (&tot)[NV]) {
  __shared__ double sh[NV][kBlk / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    T x = v[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[a][wid] = (double)x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < kBlk / 32; ++w) s += sh[a][w];
      red.partials[blockIdx.x * 4 + a] = s;
    }
    __threadfence();
    unsigned t = atomicAdd(red.ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  // The last block adds the partials with all its threads: thread t sums
  // blocks t, t + kBlk, ... in order, then a fixed-shape tree; the order
  // depends only on gridDim, so the result is deterministic.
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int a = 0; a < NV; ++a) acc[a] = 0.0;
  // one pass over the partials, all NV values of a block together (the loads
  // of several blocks in flight); each sum still runs over b in order
#pragma unroll 4
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kBlk) {
    double v[NV];
#pragma unroll
    for (int a = 0; a < NV; ++a) v[a] = __ldcg(red.partials + b * 4 + a);
#pragma unroll
    for (int a = 0; a < NV; ++a) acc[a] += v[a];
  }
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    double s = acc[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh[a][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < kBlk / 32; ++w) s += sh[a][w];
      tot[a] = s;
    }
    *red.ticket = 0u;
  }
  return threadIdx.x == 0;
}

// ------------------------------------------------------------------ SELL SpMV
// y = A x over all slices (one warp per slice, lane = row).  Returns the
// thread's partial of y.w (w = x when wdot is null); with rdot, also adds
// rdot.x into *part2.
template <typename T, bool D16, bool DIFF = false>
__device__ __forceinline__ T sell_rows(const SellView& A, const T* __restrict__ v, const T* __restrict__ x,
                                            T* __restrict__ y, const T* __restrict__ wdot,
                                            const T* __restrict__ rdot = nullptr, T* part2 = nullptr) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * kBlk + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * kBlk) >> 5;
  T part = 0;
  for (int64_t s = warp; s < A.nslices; s += nwarps) {
    const int64_t row = s * 32 + lane;
    const T xi = (DIFF && row < A.nrows) ? x[row] : (T)0;
    const T acc = sell_row_acc<T, D16, DIFF>(A, v, x, s, lane, xi);
    if (row < A.nrows) {
      y[row] = acc;
      const T xr = x[row];
      part += acc * (wdot ? wdot[row] : xr);
      if (rdot) *part2 += rdot[row] * xr;
    }
  }
  return part;
}

// CG: q = A p, scal[slot] = p.q, alpha.  Skips a finished or paused iteration.
// Standard CG: alpha = r.z / p.Ap.  FLEX (flexible CG, used by the FP32
// refinement): alpha = r.p / p.Ap, the step that minimises the energy error
// along p even when r is not orthogonal to the previous direction -- as after
// a residual replacement; equal to the standard step in exact arithmetic.
template <typename T, bool D16, bool DIFF, bool FLEX>
__global__ void __launch_bounds__(kBlk, sell_occ<T>()) sell_cg_spmv_k(SellView A, const T* __restrict__ v, const T* __restrict__ x,
                                                      T* __restrict__ y, const T* __restrict__ r, Red4 red,
                                                      double* scal, int slot, int* flags) {
  pdl_launch_dependents();
  pdl_wait();
  if (flags[F_DONE] || flags[F_RU]) {
    // F_RU = 1: requested by the previous update; p has been advanced once by
    // cg_p_k since.  Mark it 2 so the rest of the graph skips until the host
    // has replaced the residual.
    if (flags[F_RU] == 1 && blockIdx.x == 0 && threadIdx.x == 0) ((volatile int*)flags)[F_RU] = 2;
    return;
  }
  T rp = 0;
  T p[2];
  p[0] = sell_rows<T, D16, DIFF>(A, v, x, y, nullptr, FLEX ? r : nullptr, &rp);
  p[1] = rp;
  double t[2];
  if (grid_sums<2>(p, red, t)) {
    const double pq = t[0];
    scal[slot] = pq;
    const double num = FLEX ? t[1] : scal[S_RZ];
    scal[S_ALPHA] = (pq > 0.0 && isfinite(pq)) ? num / pq : 0.0;
  }
}

// r = b - A x in FP64 (permuted order), scal[slot] = r.r
template <bool D16>
__global__ void __launch_bounds__(kBlk, kSellOcc) sell_resid_k(SellView A, const double* __restrict__ v,
                                                    const double* __restrict__ x, const double* __restrict__ b,
                                                    double* __restrict__ r, Red4 red, double* scal, int slot) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * kBlk + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * kBlk) >> 5;
  double part = 0.0;
  for (int64_t s = warp; s < A.nslices; s += nwarps) {
    const int64_t row = s * 32 + lane;
    const double acc = sell_row_resid<D16>(A, v, x, s, lane);
    if (row < A.nrows) {
      const double rv = b[row] - acc;
      r[row] = rv;
      part += rv * rv;
    }
  }
  double p[1] = {part};
  double t[1];
  if (grid_sums<1>(p, red, t)) scal[slot] = t[0];
}

// CSR (original order): r = b - A_ff x - A_fd t, rr partial; for the lifted
// right-hand side and the final residual.  t may be null (no data columns).
template <int G>
__global__ void __launch_bounds__(kBlk) resid64_k(int64_t n, const int32_t* __restrict__ rp,
                                                 const int32_t* __restrict__ ci, const double* __restrict__ v,
                                                 const double* __restrict__ x, const int32_t* __restrict__ rpd,
                                                 const int32_t* __restrict__ cid, const double* __restrict__ vd,
                                                 const double* __restrict__ t, int64_t nu,
                                                 const double* __restrict__ b, double* __restrict__ r, Red4 red,
                                                 double* scal, int slot) {
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int g = lane / G, lg = lane % G;
  const int64_t warp = ((int64_t)blockIdx.x * kBlk + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * kBlk) >> 5;
  double part = 0.0;
  for (int64_t r0 = warp * RPW; r0 < n; r0 += nwarps * RPW) {
    const int64_t row = r0 + g;
    double s = 0.0;
    if (row < n) {
      const int32_t bb = rp[row], e = rp[row + 1];
      for (int32_t k = bb + lg; k < e; k += G) s += v[k] * x[ci[k]];
      if (t) {
        const int32_t bd = rpd[row], ed = rpd[row + 1];
        for (int32_t k = bd + lg; k < ed; k += G) s += vd[k] * t[cid[k] - nu];
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    if (row < n && lg == 0) {
      const double rv = b[row] - s;
      r[row] = rv;
      part += rv * rv;
    }
  }
  double p[1] = {part};
  double tt[1];
  if (grid_sums<1>(p, red, tt)) scal[slot] = tt[0];
}

// ------------------------------------------------------------------ PCG
// Grid-stride loops process 4 items per thread per step (independent loads in
// flight).
#define FOR4(i, n)                                                                                \
  for (int64_t i##0 = blockIdx.x * (int64_t)kBlk + threadIdx.x, i##s = (int64_t)gridDim.x * kBlk; \
       i##0 < (n); i##0 += 4 * i##s)                                                              \
    _Pragma("unroll") for (int i##u = 0; i##u < 4; ++i##u)                                        \
      if (const int64_t i = i##0 + i##u * i##s; i < (n))

template <typename T, bool ACC>
__global__ void __launch_bounds__(kBlk, kVecOcc) cg_update_k(int64_t n, T* __restrict__ x, T* __restrict__ r,
                                                   const T* __restrict__ p, const T* __restrict__ q,
                                                   T* __restrict__ z, const T* __restrict__ dinv, Red4 red,
                                                   double* scal, int* flags) {
  pdl_launch_dependents();
  pdl_wait();
  if (flags[F_DONE] || flags[F_RU]) return;
  // breakdown (p.Ap not positive or not finite): no update, report below
  const double pq = scal[S_PQ];
  const bool brk = !(pq > 0.0) || !isfinite(pq);
  const T alpha = brk ? (T)0 : (T)scal[S_ALPHA];
  T prz = 0, prr = 0, pzo = 0;
  FOR4(i, n) {
    const T pi = p[i];
    x[i] += alpha * pi;
    const T ro = r[i];
    const T ri = ro - alpha * q[i];
    r[i] = ri;
    const T zi = dinv[i] * ri;
    z[i] = zi;
    prz += ri * zi;
    prr += ri * ri;
    if (ACC) pzo += zi * ro;
  }
  T v[3] = {prz, prr, pzo};
  double t[3];
  if (grid_sums<3>(v, red, t)) {
    const double rz = t[0], rr = t[1];
    // FP32 refinement: Polak-Ribiere beta (flexible CG, Notay 2000),
    // z_new.(r_new - r_old) / (r_old.z_old); standard CG: r_new.z_new / r_old.z_old
    scal[S_BETA] = (ACC ? rz - t[2] : rz) / scal[S_RZ];
    scal[S_RZ] = rz;
    scal[S_RR] = rr;
    const int it = ++flags[F_ITER];
    const bool conv = rr <= scal[S_TOL2] * (ACC ? scal[S_BN2S] : scal[S_BN2]);
    const bool bad = brk || !isfinite(rz) || !isfinite(rr);
    if (!ACC) {
      if (conv || bad || it >= flags[F_MAXIT]) {
        flags[F_DONE] = 1;
        flags[F_CONV] = (conv && !bad) ? 1 : 0;
      }
    } else if (bad) {
      // FP32 recurrence broke down (e.g. its residual reached exactly zero):
      // replace the residual and restart the direction from it
      flags[F_BRK] = 1;
      flags[F_RU] = 1;
    } else {
      // FP32 recurrence: ask for an FP64 residual replacement when the
      // residual dropped by delta since the last one, or looks converged.
      const double rn = sqrt(rr);
      if (rn > scal[S_RMAX]) scal[S_RMAX] = rn;
      // a recurrence that looks converged has spent its search directions:
      // the replacement restarts from p = z (F_BRK = 2)
      if (conv) flags[F_BRK] = 2;
      if (conv || it >= flags[F_MAXIT] || rn < scal[S_DELTA] * scal[S_RMAX]) flags[F_RU] = 1;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kBlk, kVecOcc) cg_p_k(int64_t n, T* __restrict__ p, const T* __restrict__ z,
                                              const double* scal, const int* flags) {
  // runs once more after a replacement request (F_RU = 1), so that p is the
  // recurrence's next direction when the residual gets replaced
  pdl_launch_dependents();
  pdl_wait();
  if (flags[F_DONE] || flags[F_RU] == 2) return;
  const T beta = (T)scal[S_BETA];
  FOR4(i, n) p[i] = z[i] + beta * p[i];
}

// z = dinv r, rz = r.z, and the initial scalars.  set_p: p = z (restart);
// otherwise the kept direction is carried into the new residual units:
// p *= pscale (the FP32 refinement rescales r at every replacement).
template <typename T>
__global__ void __launch_bounds__(kBlk, kVecOcc) cg_start_k(int64_t n, const T* __restrict__ r, T* __restrict__ z,
                                                  T* __restrict__ p, const T* __restrict__ dinv, Red4 red,
                                                  double* scal, int* flags, int set_p, T pscale) {
  T prz = 0;
  FOR4(i, n) {
    const T zi = dinv[i] * r[i];
    z[i] = zi;
    if (set_p) p[i] = zi;
    else if (pscale != (T)1) p[i] *= pscale;
    prz += r[i] * zi;
  }
  T v[1] = {prz};
  double t[1];
  if (grid_sums<1>(v, red, t)) {
    scal[S_RZ] = t[0];
    flags[F_RU] = 0;
  }
}

// x64 += s * xacc, xacc = 0  (the FP32 iterate solves for the correction / s)
__global__ void fold_k(int64_t n, double* __restrict__ x, float* __restrict__ xa, double s) {
  FOR4(i, n) {
    x[i] += s * (double)xa[i];
    xa[i] = 0.0f;
  }
}

// b = a * inv_s in FP32: residuals are demoted at unit norm, so FP32 dot
// products neither underflow nor overflow whatever the scale of the problem
__global__ void demote_k(int64_t n, const double* __restrict__ a, float* __restrict__ b, double inv_s) {
  FOR4(i, n) b[i] = (float)(a[i] * inv_s);
}

__global__ void add_scaled_k(int64_t n, double* __restrict__ x, const float* __restrict__ d, double s) {
  FOR4(i, n) x[i] += s * (double)d[i];
}

// out[i] = in[perm[i]]  /  out[perm[i]] = in[i]
__global__ void permute_in_k(int64_t n, const int32_t* __restrict__ perm, const double* __restrict__ in,
                             double* __restrict__ out) {
  FOR4(i, n) out[i] = in[perm[i]];
}
__global__ void permute_out_k(int64_t n, const int32_t* __restrict__ perm, const double* __restrict__ in,
                              double* __restrict__ out) {
  FOR4(i, n) out[perm[i]] = in[i];
}

// ------------------------------------------------------------------ MINRES
// Preconditioned MINRES with diagonal M (minv = M^-1); three-term buffers are
// addressed by a rotation counter in flags[F_ROT].
//   step 1 (spmv): q = A z_j,  delta = q.z_j
//   step 2 (vec):  v_{j+1} = q - (delta/gam) v_j - (gam/gamp) v_{j-1};
//                  z_{j+1} = minv v_{j+1}; gamn^2 = z_{j+1}.v_{j+1};
//                  last block: Givens rotation scalars
//   step 3 (upd):  w_{j+1} = (z_j - a3 w_{j-1} - a2 w_j)/a1;  x += c_{j+1} eta w_{j+1}
// where z_j is the normalised z (z/gam), kept in zb[rot].
template <typename T, bool D16>
__global__ void __launch_bounds__(kBlk, sell_occ<T>()) mr_spmv_k(SellView A, const T* __restrict__ v, T* const* zb,
                                                 T* __restrict__ q, Red4 red, double* scal, const int* flags) {
  if (flags[F_DONE]) return;
  const int rot = flags[F_ROT];
  const T* z = zb[rot % 3];
  T p[1] = {sell_rows<T, D16>(A, v, z, q, nullptr)};
  double t[1];
  if (grid_sums<1>(p, red, t)) scal[S_DEL] = t[0];
}

template <typename T>
__global__ void __launch_bounds__(kBlk, kVecOcc) mr_vec_k(int64_t n, const T* __restrict__ q, T* const* vb, T* const* zb,
                                                const T* __restrict__ minv, Red4 red, double* scal, int* flags) {
  if (flags[F_DONE]) return;
  const int rot = flags[F_ROT];
  T* vj = vb[rot % 3];
  T* vjm = vb[(rot + 2) % 3];
  T* vn = vb[(rot + 1) % 3];
  T* zn = zb[(rot + 1) % 3];
  const double gam = scal[S_GAM], gamp = scal[S_GAMP];
  const T a = (T)(scal[S_DEL] / gam), bcoef = (T)(gamp > 0.0 ? gam / gamp : 0.0);
  T pz = 0;
  FOR4(i, n) {
    const T vv = q[i] - a * vj[i] - bcoef * vjm[i];
    vn[i] = vv;
    const T zz = minv[i] * vv;
    zn[i] = zz;
    pz += zz * vv;
  }
  T v[1] = {pz};
  double t[1];
  if (grid_sums<1>(v, red, t)) {
    const double gamn = sqrt(fmax(t[0], 0.0));
    const double delta = scal[S_DEL];
    const double c = scal[S_C], cp = scal[S_CP], s = scal[S_S], sp = scal[S_SP], g = scal[S_GAM];
    const double a0 = c * delta - cp * s * g;
    const double a1 = sqrt(a0 * a0 + gamn * gamn);
    const double a2 = s * delta + cp * c * g;
    const double a3 = sp * g;
    const double cn = a0 / a1, sn = gamn / a1;
    scal[S_A1] = a1;
    scal[S_A2] = a2;
    scal[S_A3] = a3;
    scal[S_CN] = cn;
    scal[S_CP] = c;
    scal[S_C] = cn;
    scal[S_SP] = s;
    scal[S_S] = sn;
    scal[S_GAMP] = g;
    scal[S_GAMN] = gamn;
  }
}

template <typename T>
__global__ void __launch_bounds__(kBlk, kVecOcc) mr_upd_k(int64_t n, T* const* zb, T* const* wb, T* __restrict__ x,
                                                double* scal, int* flags) {
  if (flags[F_DONE]) return;
  const int rot = flags[F_ROT];
  const T* z = zb[rot % 3];
  T* zn = zb[(rot + 1) % 3];
  const T* wj = wb[rot % 3];
  const T* wjm = wb[(rot + 2) % 3];
  T* wn = wb[(rot + 1) % 3];
  const double a1 = scal[S_A1];
  const T a2 = (T)scal[S_A2], a3 = (T)scal[S_A3];
  const T ia1 = (T)(1.0 / a1);
  const T ce = (T)(scal[S_CN] * scal[S_ETA]);
  const double gamn = scal[S_GAMN];
  const T ig = (T)(gamn > 0.0 ? 1.0 / gamn : 0.0);
  FOR4(i, n) {
    const T w = (z[i] - a3 * wjm[i] - a2 * wj[i]) * ia1;
    wn[i] = w;
    x[i] += ce * w;
    zn[i] *= ig;  // normalise the next z for the next step
  }
}

// Advance the MINRES scalars once all blocks of mr_upd_k are done.
__global__ void mr_tail_k(double* scal, int* flags) {
  if (flags[F_DONE]) return;
  scal[S_ETA] = -scal[S_S] * scal[S_ETA];
  scal[S_GAM] = scal[S_GAMN];
  flags[F_ROT] = flags[F_ROT] + 1;
  const int it = ++flags[F_ITER];
  const bool conv = fabs(scal[S_ETA]) <= sqrt(scal[S_TOL2]) * scal[S_ETA0];
  if (conv || it >= flags[F_MAXIT] || scal[S_GAMN] == 0.0) {
    flags[F_DONE] = 1;
    flags[F_CONV] = (conv || scal[S_GAMN] == 0.0) ? 1 : 0;
  }
}

// MINRES start: v1 = r (in vb[0]), z1 = minv r, gam = sqrt(z.v).
template <typename T>
__global__ void __launch_bounds__(kBlk, kVecOcc) mr_start_k(int64_t n, const T* __restrict__ r, T* const* vb, T* const* zb,
                                                  T* const* wb, const T* __restrict__ minv, T* __restrict__ x,
                                                  Red4 red, double* scal, int* flags) {
  T pz = 0;
  FOR4(i, n) {
    const T ri = r[i];
    vb[0][i] = ri;
    vb[1][i] = 0;
    vb[2][i] = 0;
    wb[0][i] = 0;
    wb[1][i] = 0;
    wb[2][i] = 0;
    const T zi = minv[i] * ri;
    zb[0][i] = zi;
    pz += zi * ri;
    x[i] = 0;
  }
  T v[1] = {pz};
  double t[1];
  if (grid_sums<1>(v, red, t)) {
    const double g = sqrt(fmax(t[0], 0.0));
    scal[S_GAM] = g;
    scal[S_GAMP] = 0.0;
    scal[S_ETA] = g;
    scal[S_ETA0] = g;
    scal[S_C] = 1.0;
    scal[S_CP] = 1.0;
    scal[S_S] = 0.0;
    scal[S_SP] = 0.0;
    flags[F_ROT] = 0;
    flags[F_ITER] = 0;
    flags[F_DONE] = g == 0.0 ? 1 : 0;
    flags[F_CONV] = g == 0.0 ? 1 : 0;
  }
}

// z1 /= gam (after mr_start_k)
template <typename T>
__global__ void scale_k(int64_t n, T* const* zb, const double* scal) {
  const double g = scal[S_GAM];
  const T ig = (T)(g > 0.0 ? 1.0 / g : 0.0);
  FOR4(i, n) zb[0][i] *= ig;
}

// ------------------------------------------------------------------ setup
__global__ void split_count_k(int64_t nu, const int64_t* rowptr, const int32_t* col, int32_t* nff, int32_t* nfd) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nu; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t a = 0, b = 0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) (col[k] < nu) ? ++a : ++b;
    nff[r] = a;
    nfd[r] = b;
  }
}

__global__ void split_copy_k(int64_t nu, const int64_t* rowptr, const int32_t* col, const int32_t* cptr,
                             const int32_t* contrib, const int64_t* pff, const int64_t* pfd, int32_t* cff,
                             int32_t* mff, int32_t* cfd, int32_t* mfd) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nu; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t a = pff[r], b = pfd[r];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      const int32_t cc = col[k];
      const int32_t src = contrib[cptr[k]];
      if (cc < nu) { cff[a] = cc; mff[a] = src; ++a; }
      else { cfd[b] = cc; mfd[b] = src; ++b; }
    }
  }
}

__global__ void col_of_k(const int64_t* colptr, int64_t ncol, int32_t* colof) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ncol; j += (int64_t)gridDim.x * blockDim.x)
    for (int64_t k = colptr[j]; k < colptr[j + 1]; ++k) colof[k] = (int32_t)j;
}

__global__ void to32_k(int64_t n, const int64_t* a, int32_t* b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (int32_t)a[i];
}

// Sort the rows of each window of kSigma rows by length, longest first
// (ties by row number): one 256-thread block per window, bitonic network.
__global__ void __launch_bounds__(kSigma) sigma_sort_k(int64_t nu, const int32_t* __restrict__ rowptr,
                                                      int32_t* __restrict__ perm) {
  __shared__ unsigned long long key[kSigma];
  const int64_t r = (int64_t)blockIdx.x * kSigma + threadIdx.x;
  if (r < nu) {
    const unsigned len = (unsigned)(rowptr[r + 1] - rowptr[r]);
    key[threadIdx.x] = ((unsigned long long)(0x7fffffffu - len) << 32) | (unsigned long long)(unsigned)r;
  } else {
    key[threadIdx.x] = ~0ull;
  }
  __syncthreads();
  for (int size = 2; size <= kSigma; size <<= 1) {
    const int h = size >> 1;
    if (threadIdx.x < kSigma / 2) {
      const int t = threadIdx.x;
      const int i = (t / h) * size + (t % h);
      const int j = (t / h) * size + size - 1 - (t % h);
      const unsigned long long a = key[i], b = key[j];
      if (a > b) { key[i] = b; key[j] = a; }
    }
    __syncthreads();
    for (int stride = h >> 1; stride > 0; stride >>= 1) {
      if (threadIdx.x < kSigma / 2) {
        const int t = threadIdx.x;
        const int i = (t / stride) * 2 * stride + (t % stride);
        const int j = i + stride;
        const unsigned long long a = key[i], b = key[j];
        if (a > b) { key[i] = b; key[j] = a; }
      }
      __syncthreads();
    }
  }
  if (r < nu) perm[r] = (int32_t)(key[threadIdx.x] & 0xffffffffull);
}

__global__ void iperm_k(int64_t nu, const int32_t* perm, int32_t* iperm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nu; i += (int64_t)gridDim.x * blockDim.x)
    iperm[perm[i]] = (int32_t)i;
}

// slice width = length of its first (longest) row; w32[s] = 32 * width (for the scan)
__global__ void slice_width_k(int64_t nu, int64_t nsl, const int32_t* rowptr, const int32_t* perm, int32_t* sw,
                              int32_t* w32) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nsl; s += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = perm[s * 32];
    const int32_t w = rowptr[r + 1] - rowptr[r];
    sw[s] = w;
    w32[s] = 32 * w;
  }
}

// Fill one permuted row per thread; padding: map = -1, column = own row.
__global__ void sell_fill_k(int64_t nu, int64_t nsl, const int32_t* __restrict__ rowptr,
                            const int32_t* __restrict__ colff, const int32_t* __restrict__ mapff,
                            const int32_t* __restrict__ perm, const int32_t* __restrict__ iperm,
                            const int64_t* __restrict__ sptr, const int32_t* __restrict__ sw, int32_t* __restrict__ col,
                            int32_t* __restrict__ map, int* __restrict__ wide) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nsl * 32;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = i >> 5;
    const int lane = (int)(i & 31);
    const int64_t base = sptr[s] + lane;
    const int w = sw[s];
    int len = 0;
    int32_t rp = 0;
    if (i < nu) {
      const int32_t r = perm[i];
      rp = rowptr[r];
      len = rowptr[r + 1] - rp;
    }
    for (int j = 0; j < w; ++j) {
      const int64_t k = base + (int64_t)j * 32;
      if (j < len) {
        const int32_t cn = iperm[colff[rp + j]];
        col[k] = cn;
        map[k] = mapff[rp + j];
        const int64_t d = (int64_t)cn - i;
        if (d < -32768 || d > 32767) atomicExch(wide, 1);
      } else {
        col[k] = i < nu ? (int32_t)i : 0;
        map[k] = -1;
      }
    }
  }
}

__global__ void sell_delta_k(int64_t npad, int64_t nu, const int64_t* sptr, int64_t nsl, const int32_t* col,
                             int16_t* dcol) {
  // entry k of slice s, lane l belongs to row s*32 + l; slices are contiguous
  for (int64_t s = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5); s < nsl;
       s += (int64_t)gridDim.x * (blockDim.x / 32)) {
    const int lane = threadIdx.x & 31;
    const int64_t row = s * 32 + lane;
    for (int64_t k = sptr[s] + lane; k < sptr[s + 1]; k += 32)
      dcol[k] = (int16_t)(row < nu ? (int64_t)col[k] - row : 0);
  }
}

__global__ void sell_vals_k(int64_t npad, const int32_t* __restrict__ map, const double* __restrict__ vals,
                            double* __restrict__ v64, float* __restrict__ v32) {
  FOR4(k, npad) {
    const int32_t m = map[k];
    const double v = m >= 0 ? vals[m] : 0.0;
    v64[k] = v;
    v32[k] = (float)v;
  }
}

// FP32 values in difference form: each row's diagonal slot gets the row sum
// s_i = sum_j a_ij (added in FP64, rounded once); the other slots keep a_ij.
template <bool D16>
__global__ void sell_rowsum_k(SellView A, const int32_t* __restrict__ map, const double* __restrict__ v64,
                              float* __restrict__ v32) {
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < A.nrows;
       row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = row >> 5;
    const int64_t base = A.sptr[s] + (row & 31);
    const int w = A.sw[s];
    double sum = 0.0;
    int64_t dpos = -1;
    for (int j = 0; j < w; ++j) {
      const int64_t k = base + (int64_t)j * 32;
      if (map[k] < 0) continue;  // padding
      sum += v64[k];
      const int c = D16 ? (int)row + (int)A.d16[k] : A.c32[k];
      if ((int64_t)c == row) dpos = k;
    }
    if (dpos >= 0) v32[dpos] = (float)sum;
  }
}

__global__ void gather_vals_k(int64_t n, const int32_t* map, const double* src, double* d64) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d64[i] = src[map[i]];
}

// Preconditioner diagonal in the original order: 1/K_ii where K_ii != 0, else
// 1/aux_i where aux_i > 0 (pressure mass diagonal), else 1.  abs_diag selects
// |K_ii| (MINRES needs an SPD preconditioner).
__global__ void diag_k(int64_t nu, const int32_t* rp, const int32_t* ci, const double* v, const double* aux,
                       int abs_diag, double* d) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nu; r += (int64_t)gridDim.x * blockDim.x) {
    double dv = 0.0;
    int32_t lo = rp[r], hi = rp[r + 1] - 1;
    while (lo <= hi) {
      int32_t mid = (lo + hi) >> 1;
      if (ci[mid] == r) { dv = v[mid]; break; }
      if (ci[mid] < r) lo = mid + 1; else hi = mid - 1;
    }
    if (abs_diag) dv = fabs(dv);
    double inv;
    if (dv != 0.0) inv = 1.0 / dv;
    else if (aux && aux[r] > 0.0) inv = 1.0 / aux[r];
    else inv = 1.0;
    d[r] = inv;
  }
}

__global__ void permute_diag_k(int64_t n, const int32_t* perm, const double* in, double* d64, float* d32) {
  FOR4(i, n) {
    const double v = in[perm[i]];
    d64[i] = v;
    d32[i] = (float)v;
  }
}

static int pick_group(int64_t nnz, int64_t n) {
  const double avg = n > 0 ? (double)nnz / (double)n : 0.0;
  if (avg <= 3) return 2;
  if (avg <= 10) return 4;
  if (avg <= 24) return 8;
  if (avg <= 48) return 16;
  return 32;
}

static unsigned vec_grid(int64_t n) { return grid_for(n, kBlk * 4, kVecGridCap); }
// one full wave of the kernel's resident blocks: no ragged second wave
template <typename T = double>
static unsigned sell_grid(const SolverData* S) {
  return grid_for(S->A.nslices, kBlk / 32, (int64_t)152 * sell_occ<T>());
}

static Red4 red_area(SolverData* S, int k) {
  Red4 r;
  r.partials = S->red.p + (size_t)k * kMaxRedBlocks * 4;
  r.ticket = S->tickets.p + k;
  return r;
}

static int build_sell(Ctx* c, SolverData* S) {
  const int64_t nu = S->nu;
  Sell& A = S->A;
  A.nrows = nu;
  A.nslices = (nu + 31) / 32;
  const int64_t nsl = A.nslices;
  const int64_t nwin = (nu + kSigma - 1) / kSigma;
  DBuf<int32_t> iperm, w32, col;
  DBuf<int> wide;
  ELFEL_TRY(A.perm.alloc(c, (size_t)nsl * 32));
  ELFEL_TRY(iperm.alloc(c, (size_t)(nu > 0 ? nu : 1)));
  // rows past nu in the last slice map to row 0 (never written)
  ELFEL_CUDA(c, cudaMemsetAsync(A.perm.p, 0, sizeof(int32_t) * nsl * 32, c->stream));
  sigma_sort_k<<<(unsigned)nwin, kSigma, 0, c->stream>>>(nu, S->ff.rowptr.p, A.perm.p);
  iperm_k<<<grid_for(nu, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(nu, A.perm.p, iperm.p);
  ELFEL_LAUNCH_CHECK(c);
  ELFEL_TRY(A.sw.alloc(c, (size_t)nsl));
  ELFEL_TRY(w32.alloc(c, (size_t)nsl));
  ELFEL_TRY(A.sptr.alloc(c, (size_t)nsl + 1));
  slice_width_k<<<grid_for(nsl, 256), 256, 0, c->stream>>>(nu, nsl, S->ff.rowptr.p, A.perm.p, A.sw.p, w32.p);
  ELFEL_LAUNCH_CHECK(c);
  ELFEL_TRY(scan_counts_i32(c, w32.p, nsl, A.sptr.p));
  w32.release(c);
  ELFEL_CUDA(c, cudaMemcpyAsync(&A.nnz_pad, A.sptr.p + nsl, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  if (A.nnz_pad >= (int64_t)0x7fffffff) return fail(c, ELFEL_ERR_ARG, "solver matrix too large for 32-bit offsets");
  const size_t np = (size_t)(A.nnz_pad > 0 ? A.nnz_pad : 1);
  ELFEL_TRY(col.alloc(c, np));
  ELFEL_TRY(A.map.alloc(c, np));
  ELFEL_TRY(wide.alloc(c, 1));
  ELFEL_CUDA(c, cudaMemsetAsync(wide.p, 0, sizeof(int), c->stream));
  sell_fill_k<<<grid_for(nsl * 32, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
      nu, nsl, S->ff.rowptr.p, S->ff.col.p, S->ff.map.p, A.perm.p, iperm.p, A.sptr.p, A.sw.p, col.p, A.map.p, wide.p);
  ELFEL_LAUNCH_CHECK(c);
  int hw = 0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&hw, wide.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  wide.release(c);
  iperm.release(c);
  if (!hw) {
    A.d16 = 1;
    ELFEL_TRY(A.dcol.alloc(c, np));
    sell_delta_k<<<grid_for(nsl, 8, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(A.nnz_pad, nu, A.sptr.p, nsl,
                                                                                    col.p, A.dcol.p);
    ELFEL_LAUNCH_CHECK(c);
    col.release(c);
  } else {
    A.d16 = 0;
    A.col = col;
    col.p = nullptr;
    col.n = 0;
  }
  ELFEL_TRY(A.v64.alloc(c, np));
  ELFEL_TRY(A.v32.alloc(c, np));
  return ELFEL_OK;
}

int build_solver(elfel_sysmat* m, int64_t nu) {
  Ctx* c = &m->h->c;
  if (!m->solver) m->solver = new SolverData();
  SolverData* S = m->solver;
  if (S->nu == nu && S->pattern_id == (const void*)m->P.rowval.p && S->pattern_nnz == m->P.nnz) return ELFEL_OK;
  S->release(c);
  Phase ph(c, "solver_setup");
  const int64_t n = m->nrow;
  // Full CSR of K through the pattern builder: slots = CSC nonzeros, with
  // row and column roles swapped so that the CSC of K^T (= CSR of K) comes out.
  DBuf<int32_t> colof;
  ELFEL_TRY(colof.alloc(c, (size_t)(m->P.nnz > 0 ? m->P.nnz : 1)));
  if (m->P.ncol > 0) {
    col_of_k<<<grid_for(m->P.ncol, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(m->P.colptr.p, m->P.ncol,
                                                                                        colof.p);
    ELFEL_LAUNCH_CHECK(c);
  }
  SlotGen g;
  g.I = colof.p;        // "row" of the transposed matrix = column of K
  g.J = m->P.rowval.p;  // "column" of the transposed matrix = row of K
  g.ncoo = m->P.nnz;
  Pattern R;
  ELFEL_TRY(build_pattern(c, g, m->ncol, m->nrow, &R));
  colof.release(c);
  // split the first nu rows into free (col < nu) and data (col >= nu) parts
  DBuf<int32_t> nff, nfd;
  DBuf<int64_t> pff, pfd;
  ELFEL_TRY(nff.alloc(c, (size_t)nu + 1));
  ELFEL_TRY(nfd.alloc(c, (size_t)nu + 1));
  ELFEL_TRY(pff.alloc(c, (size_t)nu + 1));
  ELFEL_TRY(pfd.alloc(c, (size_t)nu + 1));
  const unsigned gr = grid_for(nu, 256, (int64_t)c->sm_count * 16);
  if (nu > 0) {
    split_count_k<<<gr, 256, 0, c->stream>>>(nu, R.colptr.p, R.rowval.p, nff.p, nfd.p);
    ELFEL_LAUNCH_CHECK(c);
  }
  ELFEL_TRY(scan_counts_i32(c, nff.p, nu, pff.p));
  ELFEL_TRY(scan_counts_i32(c, nfd.p, nu, pfd.p));
  int64_t tff = 0, tfd = 0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&tff, pff.p + nu, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(&tfd, pfd.p + nu, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  S->ff.nrows = S->fd.nrows = nu;
  S->ff.nnz = tff;
  S->fd.nnz = tfd;
  ELFEL_TRY(S->ff.rowptr.alloc(c, (size_t)nu + 1));
  ELFEL_TRY(S->fd.rowptr.alloc(c, (size_t)nu + 1));
  ELFEL_TRY(S->ff.col.alloc(c, (size_t)(tff > 0 ? tff : 1)));
  ELFEL_TRY(S->ff.map.alloc(c, (size_t)(tff > 0 ? tff : 1)));
  ELFEL_TRY(S->fd.col.alloc(c, (size_t)(tfd > 0 ? tfd : 1)));
  ELFEL_TRY(S->fd.map.alloc(c, (size_t)(tfd > 0 ? tfd : 1)));
  ELFEL_TRY(S->ff.v64.alloc(c, (size_t)(tff > 0 ? tff : 1)));
  ELFEL_TRY(S->fd.v64.alloc(c, (size_t)(tfd > 0 ? tfd : 1)));
  to32_k<<<grid_for(nu + 1, 256), 256, 0, c->stream>>>(nu + 1, pff.p, S->ff.rowptr.p);
  to32_k<<<grid_for(nu + 1, 256), 256, 0, c->stream>>>(nu + 1, pfd.p, S->fd.rowptr.p);
  if (nu > 0)
    split_copy_k<<<gr, 256, 0, c->stream>>>(nu, R.colptr.p, R.rowval.p, R.cptr.p, R.contrib.p, pff.p, pfd.p,
                                            S->ff.col.p, S->ff.map.p, S->fd.col.p, S->fd.map.p);
  ELFEL_LAUNCH_CHECK(c);
  R.release(c);
  nff.release(c); nfd.release(c); pff.release(c); pfd.release(c);
  S->nu = nu;
  if (nu > 0) ELFEL_TRY(build_sell(c, S));
  const size_t vn = (size_t)(nu > 0 ? nu : 1);
  for (DBuf<double>* b : {&S->bo64, &S->xo64, &S->ro64, &S->dinvo, &S->dinv64, &S->b64, &S->x64, &S->r64, &S->z64,
                          &S->p64, &S->q64, &S->y64})
    ELFEL_TRY(b->alloc(c, vn));
  for (DBuf<float>* b : {&S->dinv32, &S->r32, &S->p32, &S->q32, &S->z32, &S->xa32, &S->zz32, &S->b32, &S->x32})
    ELFEL_TRY(b->alloc(c, vn));
  ELFEL_TRY(S->T64.alloc(c, (size_t)(n > 0 ? n : 1)));
  ELFEL_TRY(S->scal.alloc(c, S_COUNT));
  ELFEL_TRY(S->flags.alloc(c, F_COUNT));
  ELFEL_TRY(S->red.alloc(c, (size_t)3 * kMaxRedBlocks * 4));
  ELFEL_TRY(S->tickets.alloc(c, 4));
  ELFEL_CUDA(c, cudaMemsetAsync(S->tickets.p, 0, sizeof(unsigned) * 4, c->stream));
  ELFEL_CUDA(c, cudaMemsetAsync(S->scal.p, 0, sizeof(double) * S_COUNT, c->stream));
  ELFEL_CUDA(c, cudaMemsetAsync(S->flags.p, 0, sizeof(int) * F_COUNT, c->stream));
  S->group = pick_group(tff, nu);
  S->pattern_id = m->P.rowval.p;
  S->pattern_nnz = m->P.nnz;
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  return ELFEL_OK;
}

// Values of the solver matrices from the CSC values (FP64, and the FP32 copy).
// diff32: the FP32 copy is stored in difference form (for the FP32 CG).
int refresh_values(elfel_sysmat* m, int abs_diag, int diff32) {
  Ctx* c = &m->h->c;
  SolverData* S = m->solver;
  const int64_t nu = S->nu;
  Phase ph(c, "solver_values");
  if (S->ff.nnz)
    gather_vals_k<<<grid_for(S->ff.nnz, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
        S->ff.nnz, S->ff.map.p, m->vals.p, S->ff.v64.p);
  if (S->fd.nnz)
    gather_vals_k<<<grid_for(S->fd.nnz, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
        S->fd.nnz, S->fd.map.p, m->vals.p, S->fd.v64.p);
  if (S->A.nnz_pad)
    sell_vals_k<<<vec_grid(S->A.nnz_pad), kBlk, 0, c->stream>>>(S->A.nnz_pad, S->A.map.p, m->vals.p, S->A.v64.p,
                                                                 S->A.v32.p);
  if (diff32 && nu > 0) {
    const SellView V = S->view();
    if (S->A.d16)
      sell_rowsum_k<true><<<grid_for(nu, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
          V, S->A.map.p, S->A.v64.p, S->A.v32.p);
    else
      sell_rowsum_k<false><<<grid_for(nu, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
          V, S->A.map.p, S->A.v64.p, S->A.v32.p);
  }
  const double* aux = (m->fused && m->F.physics == ELFEL_STOKES) ? m->F.pmass_diag.p : nullptr;
  if (nu > 0) {
    diag_k<<<grid_for(nu, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(nu, S->ff.rowptr.p, S->ff.col.p,
                                                                                S->ff.v64.p, aux, abs_diag,
                                                                                S->dinvo.p);
    permute_diag_k<<<vec_grid(nu), kBlk, 0, c->stream>>>(nu, S->A.perm.p, S->dinvo.p, S->dinv64.p, S->dinv32.p);
  }
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

// CSR residual in the original order: r = b - A_ff x (- A_fd t); scal[slot] = r.r
static int launch_resid(Ctx* c, SolverData* S, const double* x, const double* t, const double* b, double* r,
                        Red4 red, int slot) {
  const unsigned grid = grid_for(S->nu * S->group, kBlk, kGridCap);
  const int64_t n = S->nu;
  const Csr &A = S->ff, &D = S->fd;
#define RES_ARGS \
  n, A.rowptr.p, A.col.p, A.v64.p, x, D.rowptr.p, D.col.p, D.v64.p, t, S->nu, b, r, red, S->scal.p, slot
  switch (S->group) {
    case 2: resid64_k<2><<<grid, kBlk, 0, c->stream>>>(RES_ARGS); break;
    case 4: resid64_k<4><<<grid, kBlk, 0, c->stream>>>(RES_ARGS); break;
    case 8: resid64_k<8><<<grid, kBlk, 0, c->stream>>>(RES_ARGS); break;
    case 16: resid64_k<16><<<grid, kBlk, 0, c->stream>>>(RES_ARGS); break;
    default: resid64_k<32><<<grid, kBlk, 0, c->stream>>>(RES_ARGS); break;
  }
#undef RES_ARGS
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

// SELL residual in the permuted order (FP64).
static int launch_sell_resid(Ctx* c, SolverData* S, const double* x, const double* b, double* r, Red4 red, int slot) {
  const SellView V = S->view();
  if (S->A.d16)
    sell_resid_k<true><<<sell_grid(S), kBlk, 0, c->stream>>>(V, S->A.v64.p, x, b, r, red, S->scal.p, slot);
  else
    sell_resid_k<false><<<sell_grid(S), kBlk, 0, c->stream>>>(V, S->A.v64.p, x, b, r, red, S->scal.p, slot);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

// DIFF: the values are in difference form (row sums in the diagonal slots);
// FLEX: flexible-CG step length (needs the residual r).
template <typename T, bool DIFF, bool FLEX>
static void launch_cg_spmv(Ctx* c, SolverData* S, const T* v, const T* x, T* y, const T* r, Red4 red, int slot) {
  const SellView V = S->view();
  if (S->A.d16)
    launch_pdl(sell_cg_spmv_k<T, true, DIFF, FLEX>, sell_grid<T>(S), kBlk, c->stream, V, v, x, y, r, red, S->scal.p,
               slot, S->flags.p);
  else
    launch_pdl(sell_cg_spmv_k<T, false, DIFF, FLEX>, sell_grid<T>(S), kBlk, c->stream, V, v, x, y, r, red, S->scal.p,
               slot, S->flags.p);
}

template <typename T>
static void launch_mr_spmv(Ctx* c, SolverData* S, const T* v, T* const* zb, T* q, Red4 red) {
  const SellView V = S->view();
  if (S->A.d16)
    mr_spmv_k<T, true><<<sell_grid<T>(S), kBlk, 0, c->stream>>>(V, v, zb, q, red, S->scal.p, S->flags.p);
  else
    mr_spmv_k<T, false><<<sell_grid<T>(S), kBlk, 0, c->stream>>>(V, v, zb, q, red, S->scal.p, S->flags.p);
}

static int read_flags(Ctx* c, SolverData* S, int* h) {
  ELFEL_CUDA(c, cudaMemcpyAsync(h, S->flags.p, sizeof(int) * F_COUNT, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  return ELFEL_OK;
}

static int set_scal(Ctx* c, SolverData* S, int idx, double v) {
  ELFEL_CUDA(c, cudaMemcpyAsync(S->scal.p + idx, &v, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  return ELFEL_OK;
}

// Capture kGraphIters iterations of a kernel sequence into an executable graph.
template <typename F>
static int capture(Ctx* c, cudaGraphExec_t* out, F&& body) {
  if (*out) return ELFEL_OK;
  cudaGraph_t g;
  ELFEL_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < kGraphIters; ++k) body();
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (e != cudaSuccess) return fail(c, ELFEL_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(c, ELFEL_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return ELFEL_OK;
}

int lift_rhs(elfel_sysmat* m, const double* Fh, const double* T, int t_dev) {
  Ctx* c = &m->h->c;
  SolverData* S = m->solver;
  const int64_t n = m->nrow, nu = S->nu;
  ELFEL_CUDA(c, cudaMemcpyAsync(S->T64.p, T, sizeof(double) * n,
                                t_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  double* Fd = m->rhs.p;
  DBuf<double> Ftmp;
  if (Fh) {
    ELFEL_TRY(Ftmp.alloc(c, (size_t)n));
    ELFEL_CUDA(c, cudaMemcpyAsync(Ftmp.p, Fh, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    Fd = Ftmp.p;
  }
  ELFEL_TRY(launch_resid(c, S, S->T64.p, S->T64.p + nu, Fd, S->bo64.p, red_area(S, 2), S_BN2));
  Ftmp.release(c);
  permute_in_k<<<vec_grid(nu), kBlk, 0, c->stream>>>(nu, S->A.perm.p, S->bo64.p, S->b64.p);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

int solution_residual(elfel_sysmat* m) {
  Ctx* c = &m->h->c;
  SolverData* S = m->solver;
  const int64_t nu = S->nu;
  permute_out_k<<<vec_grid(nu), kBlk, 0, c->stream>>>(nu, S->A.perm.p, S->x64.p, S->xo64.p);
  ELFEL_LAUNCH_CHECK(c);
  return launch_resid(c, S, S->xo64.p, nullptr, S->bo64.p, S->ro64.p, red_area(S, 2), S_RR);
}

// ------------------------------------------------------------------ drivers
static int run_pcg64(elfel_sysmat* m, int maxit, elfel_solve_stats* st) {
  Ctx* c = &m->h->c;
  SolverData* S = m->solver;
  const int64_t nu = S->nu;
  const unsigned vg = vec_grid(nu);
  ELFEL_CUDA(c, cudaMemsetAsync(S->x64.p, 0, sizeof(double) * nu, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(S->r64.p, S->b64.p, sizeof(double) * nu, cudaMemcpyDeviceToDevice, c->stream));
  int hf[F_COUNT] = {0, 0, 0, maxit, 0, 0, 0};
  ELFEL_CUDA(c, cudaMemcpyAsync(S->flags.p, hf, sizeof(hf), cudaMemcpyHostToDevice, c->stream));
  cg_start_k<double><<<vg, kBlk, 0, c->stream>>>(nu, S->r64.p, S->z64.p, S->p64.p, S->dinv64.p, red_area(S, 0),
                                                 S->scal.p, S->flags.p, 1, 1.0);
  ELFEL_LAUNCH_CHECK(c);
  ELFEL_TRY(capture(c, &S->g_pcg64, [&]() {
    launch_cg_spmv<double, false, false>(c, S, S->A.v64.p, S->p64.p, S->q64.p, nullptr, red_area(S, 0), S_PQ);
    launch_pdl(cg_update_k<double, false>, vg, kBlk, c->stream, nu, S->x64.p, S->r64.p, S->p64.p, S->q64.p, S->z64.p,
               S->dinv64.p, red_area(S, 1), S->scal.p, S->flags.p);
    launch_pdl(cg_p_k<double>, vg, kBlk, c->stream, nu, S->p64.p, S->z64.p, S->scal.p, S->flags.p);
  }));
  // When the recurrence residual says converged, the true residual b - K x is
  // checked in FP64; if the two have drifted apart (ill-conditioned systems
  // at tight tolerances) the true residual replaces the recurrence one and
  // CG restarts from it.
  int replacements = 0;
  while (true) {
    ELFEL_CUDA(c, cudaGraphLaunch(S->g_pcg64, c->stream));
    ELFEL_TRY(read_flags(c, S, hf));
    if (!hf[F_DONE]) continue;
    if (!hf[F_CONV] || hf[F_ITER] >= maxit || replacements >= 50) break;
    ELFEL_TRY(launch_sell_resid(c, S, S->x64.p, S->b64.p, S->r64.p, red_area(S, 2), S_RR));
    double hsc[S_COUNT];
    ELFEL_CUDA(c, cudaMemcpyAsync(hsc, S->scal.p, sizeof(hsc), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    if (hsc[S_RR] <= hsc[S_TOL2] * hsc[S_BN2]) break;
    ++replacements;
    if (c->trace)
      fprintf(stderr, "[elfel pcg64] it %d: true residual %.3e above the recurrence's; restart\n", hf[F_ITER],
              sqrt(hsc[S_RR] / hsc[S_BN2]));
    hf[F_DONE] = 0;
    hf[F_CONV] = 0;
    ELFEL_CUDA(c, cudaMemcpyAsync(S->flags.p, hf, sizeof(hf), cudaMemcpyHostToDevice, c->stream));
    cg_start_k<double><<<vg, kBlk, 0, c->stream>>>(nu, S->r64.p, S->z64.p, S->p64.p, S->dinv64.p, red_area(S, 0),
                                                   S->scal.p, S->flags.p, 1, 1.0);
    ELFEL_LAUNCH_CHECK(c);
  }
  st->iterations = hf[F_ITER];
  st->refinements = replacements;
  return ELFEL_OK;
}

static int run_pcg32(elfel_sysmat* m, int maxit, elfel_solve_stats* st) {
  Ctx* c = &m->h->c;
  SolverData* S = m->solver;
  const int64_t nu = S->nu;
  const unsigned vg = vec_grid(nu);
  ELFEL_CUDA(c, cudaMemsetAsync(S->x64.p, 0, sizeof(double) * nu, c->stream));
  ELFEL_CUDA(c, cudaMemsetAsync(S->xa32.p, 0, sizeof(float) * nu, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(S->r64.p, S->b64.p, sizeof(double) * nu, cudaMemcpyDeviceToDevice, c->stream));
  // the FP32 recurrence works on r / s with s = ||b||: the initial residual
  // has unit norm whatever the scale of the problem (no FP32 under/overflow)
  double hsc0[S_COUNT];
  ELFEL_CUDA(c, cudaMemcpyAsync(hsc0, S->scal.p, sizeof(hsc0), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  const double s = sqrt(hsc0[S_BN2]);
  demote_k<<<vg, kBlk, 0, c->stream>>>(nu, S->r64.p, S->r32.p, 1.0 / s);
  ELFEL_TRY(set_scal(c, S, S_SCALE, s));
  ELFEL_TRY(set_scal(c, S, S_BN2S, 1.0));
  ELFEL_TRY(set_scal(c, S, S_RMAX, 1.0));
  int hf[F_COUNT] = {0, 0, 0, maxit, 0, 0, 0};
  ELFEL_CUDA(c, cudaMemcpyAsync(S->flags.p, hf, sizeof(hf), cudaMemcpyHostToDevice, c->stream));
  cg_start_k<float><<<vg, kBlk, 0, c->stream>>>(nu, S->r32.p, S->z32.p, S->p32.p, S->dinv32.p, red_area(S, 0),
                                                S->scal.p, S->flags.p, 1, 1.0f);
  ELFEL_LAUNCH_CHECK(c);
  ELFEL_TRY(capture(c, &S->g_pcg32, [&]() {
    launch_cg_spmv<float, true, true>(c, S, S->A.v32.p, S->p32.p, S->q32.p, S->r32.p, red_area(S, 0), S_PQ);
    launch_pdl(cg_update_k<float, true>, vg, kBlk, c->stream, nu, S->xa32.p, S->r32.p, S->p32.p, S->q32.p, S->z32.p,
               S->dinv32.p, red_area(S, 1), S->scal.p, S->flags.p);
    launch_pdl(cg_p_k<float>, vg, kBlk, c->stream, nu, S->p32.p, S->z32.p, S->scal.p, S->flags.p);
  }));
  int refinements = 0;
  int launches = 0;
  double hsc[S_COUNT];
  while (true) {
    ELFEL_CUDA(c, cudaGraphLaunch(S->g_pcg32, c->stream));
    ELFEL_TRY(read_flags(c, S, hf));
    ++launches;
    if (c->trace && (launches % 256) == 0) {
      ELFEL_CUDA(c, cudaMemcpyAsync(hsc, S->scal.p, sizeof(hsc), cudaMemcpyDeviceToHost, c->stream));
      ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
      fprintf(stderr, "[elfel pcg32] it %d recurrence %.3e rmax %.3e flags ru %d brk %d\n", hf[F_ITER],
              sqrt(hsc[S_RR]), hsc[S_RMAX], hf[F_RU], hf[F_BRK]);
    }
    if (!hf[F_RU]) continue;
    // recurrence residual before the replacement
    ELFEL_CUDA(c, cudaMemcpyAsync(hsc, S->scal.p, sizeof(hsc), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    const double rr_rec = hsc[S_RR] * s * s;  // recurrence residual, unscaled
    // FP64 residual replacement
    fold_k<<<vg, kBlk, 0, c->stream>>>(nu, S->x64.p, S->xa32.p, s);
    ELFEL_TRY(launch_sell_resid(c, S, S->x64.p, S->b64.p, S->r64.p, red_area(S, 2), S_RR));
    ELFEL_CUDA(c, cudaMemcpyAsync(hsc, S->scal.p, sizeof(hsc), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    ++refinements;
    const bool conv = hsc[S_RR] <= hsc[S_TOL2] * hsc[S_BN2];
    // keep the search direction unless the FP32 recurrence broke down or its
    // residual drifted far below the true one (then restart from p = z)
    const int restart = hf[F_BRK] || !(rr_rec > 0.0) || !(rr_rec >= 1e-6 * hsc[S_RR]) || !(hsc[S_RR] > 0.0);
    if (c->trace)
      fprintf(stderr, "[elfel pcg32] it %d replace %d: recurrence %.3e true %.3e (rel %.3e) brk %d restart %d\n",
              hf[F_ITER], refinements, sqrt(rr_rec), sqrt(hsc[S_RR]), sqrt(hsc[S_RR] / hsc[S_BN2]), hf[F_BRK],
              restart);
    if (!(hsc[S_RR] > 0.0)) {  // exact solution
      hf[F_CONV] = 1;
      break;
    }
    if (conv || hf[F_ITER] >= maxit) {
      hf[F_CONV] = conv ? 1 : 0;
      break;
    }
    if (hf[F_BRK]) {
      int z = 0;
      ELFEL_CUDA(c, cudaMemcpyAsync(S->flags.p + F_BRK, &z, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    }
    // the units stay those of the start (s = ||b||) for the whole solve, so
    // the kept direction p needs no conversion
    demote_k<<<vg, kBlk, 0, c->stream>>>(nu, S->r64.p, S->r32.p, 1.0 / s);
    cg_start_k<float><<<vg, kBlk, 0, c->stream>>>(nu, S->r32.p, S->z32.p, S->p32.p, S->dinv32.p, red_area(S, 0),
                                                  S->scal.p, S->flags.p, restart, 1.0f);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_TRY(set_scal(c, S, S_RMAX, sqrt(hsc[S_RR]) / s));
  }
  st->iterations = hf[F_ITER];
  st->refinements = refinements;
  return ELFEL_OK;
}

// MINRES on A x = b (precision T, permuted order).
template <typename T>
static int run_minres(Ctx* c, SolverData* S, const T* v, const T* minv, const T* b, T* x, T* const* vb, T* const* zb,
                      T* const* wb, T* q, double rtol, int maxit, cudaGraphExec_t* graph, int* iters, int* conv) {
  const int64_t nu = S->nu;
  const unsigned vg = vec_grid(nu);
  int hf[F_COUNT] = {0, 0, 0, maxit, 0, 0, 0};
  ELFEL_CUDA(c, cudaMemcpyAsync(S->flags.p, hf, sizeof(hf), cudaMemcpyHostToDevice, c->stream));
  ELFEL_TRY(set_scal(c, S, S_TOL2, rtol * rtol));
  mr_start_k<T><<<vg, kBlk, 0, c->stream>>>(nu, b, vb, zb, wb, minv, x, red_area(S, 0), S->scal.p, S->flags.p);
  scale_k<T><<<vg, kBlk, 0, c->stream>>>(nu, zb, S->scal.p);
  ELFEL_LAUNCH_CHECK(c);
  ELFEL_TRY(capture(c, graph, [&]() {
    launch_mr_spmv<T>(c, S, v, zb, q, red_area(S, 0));
    mr_vec_k<T><<<vg, kBlk, 0, c->stream>>>(nu, q, vb, zb, minv, red_area(S, 1), S->scal.p, S->flags.p);
    mr_upd_k<T><<<vg, kBlk, 0, c->stream>>>(nu, zb, wb, x, S->scal.p, S->flags.p);
    mr_tail_k<<<1, 1, 0, c->stream>>>(S->scal.p, S->flags.p);
  }));
  while (true) {
    ELFEL_CUDA(c, cudaGraphLaunch(*graph, c->stream));
    ELFEL_TRY(read_flags(c, S, hf));
    if (hf[F_DONE]) break;
  }
  *iters = hf[F_ITER];
  *conv = hf[F_CONV];
  return ELFEL_OK;
}

}  // namespace elfel

using namespace elfel;

extern "C" int elfel_solve(elfel_sysmat* m, const double* Fh, double* T, int64_t nu, int32_t method, double rtol,
                           int32_t maxit, elfel_solve_stats* stats) {
  if (!m || !m->h) return ELFEL_ERR_ARG;
  Ctx* c = &m->h->c;
  elfel_solve_stats st;
  memset(&st, 0, sizeof(st));
  if (!m->finished) return fail(c, ELFEL_ERR_STATE, "solve: finish! the matrix first");
  if (m->busy) return fail(c, ELFEL_ERR_STATE, "solve: the system is held by a batch slot");
  if (m->nrow != m->ncol) return fail(c, ELFEL_ERR_ARG, "solve: K must be square");
  if (nu < 0 || nu > m->nrow || !T) return fail(c, ELFEL_ERR_ARG, "solve: nu outside 0..%lld", (long long)m->nrow);
  if (!Fh && !m->has_rhs) return fail(c, ELFEL_ERR_ARG, "solve: no right-hand side");
  if (method < ELFEL_PCG64 || method > ELFEL_MINRES32_IR) return fail(c, ELFEL_ERR_ARG, "solve: unknown method");
  if (!(rtol > 0.0) || maxit < 1) return fail(c, ELFEL_ERR_ARG, "solve: rtol > 0 and maxit >= 1 required");
  cudaSetDevice(c->device);
  const auto t0 = std::chrono::steady_clock::now();
  ELFEL_TRY(build_solver(m, nu));
  SolverData* S = m->solver;
  const bool minres = method == ELFEL_MINRES64 || method == ELFEL_MINRES32_IR;
  ELFEL_TRY(refresh_values(m, minres ? 1 : 0, method == ELFEL_PCG32_IR ? 1 : 0));
  if (nu == 0) {
    if (stats) *stats = st;
    return ELFEL_OK;
  }
  // lifted right-hand side: b = F_f - K_ff T_f - K_fd T_d
  ELFEL_TRY(lift_rhs(m, Fh, T, 0));
  double bn2 = 0.0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&bn2, S->scal.p + S_BN2, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  ELFEL_TRY(set_scal(c, S, S_TOL2, rtol * rtol));
  ELFEL_TRY(set_scal(c, S, S_RMAX, sqrt(bn2)));
  // residual-replacement threshold of the FP32 refinement (tuning knob)
  double delta = 0.1;
  if (const char* e = getenv("ELFEL_RU_DELTA")) {
    const double d = atof(e);
    if (d > 0.0 && d < 1.0) delta = d;
  }
  ELFEL_TRY(set_scal(c, S, S_DELTA, delta));
  int rc = ELFEL_OK;
  if (bn2 == 0.0) {
    ELFEL_CUDA(c, cudaMemsetAsync(S->x64.p, 0, sizeof(double) * nu, c->stream));
    st.converged = 1;
  } else if (method == ELFEL_PCG64) {
    Phase ph(c, "pcg64");
    rc = run_pcg64(m, maxit, &st);
  } else if (method == ELFEL_PCG32_IR) {
    Phase ph(c, "pcg32_ir");
    rc = run_pcg32(m, maxit, &st);
  } else if (method == ELFEL_MINRES64) {
    Phase ph(c, "minres64");
    for (int i = 0; i < 3; ++i) {
      if (!S->v64[i].p) ELFEL_TRY(S->v64[i].alloc(c, (size_t)nu));
      if (!S->w64[i].p) ELFEL_TRY(S->w64[i].alloc(c, (size_t)nu));
    }
    DBuf<double*> dptr;
    ELFEL_TRY(dptr.alloc(c, 9));
    double* hp[9] = {S->v64[0].p, S->v64[1].p, S->v64[2].p, S->z64.p, S->p64.p, S->y64.p,
                     S->w64[0].p, S->w64[1].p, S->w64[2].p};
    ELFEL_CUDA(c, cudaMemcpyAsync(dptr.p, hp, sizeof(hp), cudaMemcpyHostToDevice, c->stream));
    if (S->g_minres64) {  // the pointer table is re-created each solve; rebuild the graph
      cudaGraphExecDestroy(S->g_minres64);
      S->g_minres64 = nullptr;
    }
    int it = 0, conv = 0;
    rc = run_minres<double>(c, S, S->A.v64.p, S->dinv64.p, S->b64.p, S->x64.p, dptr.p, dptr.p + 3, dptr.p + 6,
                            S->q64.p, rtol, maxit, &S->g_minres64, &it, &conv);
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    dptr.release(c);
    st.iterations = it;
  } else {
    // FP32 MINRES inside FP64 iterative refinement
    Phase ph(c, "minres32_ir");
    for (int i = 0; i < 3; ++i) {
      if (!S->v32[i].p) ELFEL_TRY(S->v32[i].alloc(c, (size_t)nu));
      if (!S->w32[i].p) ELFEL_TRY(S->w32[i].alloc(c, (size_t)nu));
    }
    DBuf<float*> dptr;
    ELFEL_TRY(dptr.alloc(c, 9));
    float* hp[9] = {S->v32[0].p, S->v32[1].p, S->v32[2].p, S->z32.p, S->p32.p, S->zz32.p,
                    S->w32[0].p, S->w32[1].p, S->w32[2].p};
    ELFEL_CUDA(c, cudaMemcpyAsync(dptr.p, hp, sizeof(hp), cudaMemcpyHostToDevice, c->stream));
    if (S->g_minres32) {
      cudaGraphExecDestroy(S->g_minres32);
      S->g_minres32 = nullptr;
    }
    const unsigned vg = vec_grid(nu);
    ELFEL_CUDA(c, cudaMemsetAsync(S->x64.p, 0, sizeof(double) * nu, c->stream));
    ELFEL_CUDA(c, cudaMemcpyAsync(S->r64.p, S->b64.p, sizeof(double) * nu, cudaMemcpyDeviceToDevice, c->stream));
    double rr = bn2;
    int total = 0, outer = 0;
    const double inner_tol = 1e-5;
    while (true) {
      const double s = sqrt(rr);  // inner solve on the unit-norm residual
      if (!(s > 0.0)) break;
      demote_k<<<vg, kBlk, 0, c->stream>>>(nu, S->r64.p, S->b32.p, 1.0 / s);
      int it = 0, conv = 0;
      rc = run_minres<float>(c, S, S->A.v32.p, S->dinv32.p, S->b32.p, S->x32.p, dptr.p, dptr.p + 3, dptr.p + 6,
                             S->q32.p, inner_tol, maxit - total, &S->g_minres32, &it, &conv);
      if (rc != ELFEL_OK) break;
      total += it;
      ++outer;
      add_scaled_k<<<vg, kBlk, 0, c->stream>>>(nu, S->x64.p, S->x32.p, s);
      ELFEL_TRY(launch_sell_resid(c, S, S->x64.p, S->b64.p, S->r64.p, red_area(S, 2), S_RR));
      ELFEL_CUDA(c, cudaMemcpyAsync(&rr, S->scal.p + S_RR, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
      if (c->trace)
        fprintf(stderr, "[elfel minres32] outer %d inner %d rel %.3e\n", outer, it, sqrt(rr / bn2));
      if (rr <= rtol * rtol * bn2 || total >= maxit || outer >= 100) break;
    }
    dptr.release(c);
    st.iterations = total;
    st.refinements = outer;
  }
  if (rc != ELFEL_OK) return rc;
  // solution back to the original order; final FP64 residual there
  ELFEL_TRY(solution_residual(m));
  double rr = 0.0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&rr, S->scal.p + S_RR, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(T, S->xo64.p, sizeof(double) * nu, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  st.relres = bn2 > 0.0 ? sqrt(rr / bn2) : 0.0;
  st.converged = st.relres <= rtol ? 1 : 0;
  st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = st;
  if (!st.converged)
    return fail(c, ELFEL_ERR_NOT_CONVERGED, "solve: relative residual %.3e > %.3e after %d iterations (%d replacements)",
                st.relres, rtol, st.iterations, st.refinements);
  return ELFEL_OK;
}
