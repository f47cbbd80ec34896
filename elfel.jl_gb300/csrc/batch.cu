// Batched solves of many systems K_m x_m = b_m (the lifted free-free systems
// of the reference's solve!, Elfel.jl test/test_heat.jl:73-76), iterated
// together: every launch works on the row tiles of all active systems.
//
// Layout.  Each system keeps its own SELL-C-sigma matrix and Krylov vectors
// (the one-system solver data).  A tile is sl * kBlk consecutive permuted
// rows of one system (sl * kBlk / 32 SELL slices; each warp works through sl
// of them and forms one partial; sl = 8 from 2M unknowns, 4 from 64k, 1
// below); a work item is a run of consecutive tiles of one system.  A device
// item map lists the items of all active systems; the three kernels of an
// iteration loop over it with a fixed grid, so one captured CUDA graph of
// kIters iterations serves any mix of systems, and systems join or leave
// between graph launches by rewriting the map.
//
// Reductions are per system and deterministic: each tile writes its partial
// sums (a fixed tree inside the tile), and the block that completes a
// system's last work item adds that system's tile partials in tile order
// with a fixed tree.  Nothing depends on which other systems share the
// launch, on how tiles are grouped into items or on the grid size, so a
// system's iterates are bit-identical alone and in any mix.
//
// Methods.  ELFEL_PCG64: Jacobi PCG in FP64.  ELFEL_PCG32_IR: Jacobi CG on the
// FP32 difference-form copy of K with FP64 residual replacement (reliable
// updates), flexible step and Polak-Ribiere beta, as the one-system driver;
// here the replacement runs on the device as a phase of the system's state
// machine, without the host:
//   M_CG       spmv: q = A p, alpha     update: x, r, z, beta     p = z + beta p
//   M_FOLD     (requested by the update) p = z + beta p; x64 += s x32; x32 = 0
//              spmv: r64 = b - K x64 in FP64; converged -> M_DONE, else M_RESTART
//   M_RESTART  update: r32 = r64 / s, z = D r32, p = z (restart) or kept
//   M_STARTED  p kernel skips; next spmv returns to M_CG
#include <math.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <vector>

#include "solve.cuh"

namespace elfel {

// per-system scalars
enum { B_RZ = 0, B_PQ, B_ALPHA, B_BETA, B_RR, B_RMAX, B_DELTA, B_TOL2, B_BN2, B_SCALE, B_RRT, B_RREC, B_COUNT = 16 };
// per-system ints
enum { I_MODE = 0, I_ITER, I_MAXIT, I_BRK, I_RESTART, I_CONV, I_REPL, I_COUNT = 8 };
enum { M_IDLE = 0, M_CG, M_FOLD, M_RESTART, M_STARTED, M_DONE };

// One system as the batched kernels see it.
struct BSys {
  SellView A;
  const float* v32;
  const double* v64;
  const float* dinv32;
  const double* dinv64;
  float *x32, *r32, *z32, *p32, *q32;
  double *x64, *r64, *z64, *p64, *q64;
  const double* b64;
  int64_t ntiles;
  int sl, pad_;        // row groups of kBlk per tile (1, 4 or 8: fixed per system by its size)
  double* part;        // ntiles x 4 partial sums
  unsigned* ticket;    // work items finished in the current kernel
  const int* nitems;   // work items of this system in the current map
  double* sc;          // B_COUNT scalars
  int* st;             // I_COUNT ints
};

constexpr int kItemMax = 32;  // tiles per work item (bounds the shared staging)
constexpr int kWarps = kBlk / 32;
// A tile: sl groups of kBlk rows; each warp accumulates its sl slices (or
// rows) in registers and reduces once, so a tile partial costs one warp
// reduction per sl * 32 rows.  sl is a property of the system (its size),
// never of the mix: large systems take more row groups (fewer reductions and
// partials), small ones fewer (no empty row groups).  Measured on the heat
// serving stream (up to about 1M unknowns) and a 4M-unknown system, 16 row
// groups were slower than 8 on both.
constexpr int kSlSmall = 1, kSlMid = 4, kSlLarge = 8;
constexpr int64_t kSlMidRows = 65536;     // unknowns from which a system takes kSlMid
constexpr int64_t kSlLargeRows = 1 << 21; // unknowns from which a system takes kSlLarge
constexpr int kTileRowsMax = kSlLarge * kBlk;

static int tile_row_groups(int64_t nu) {
  return nu >= kSlLargeRows ? kSlLarge : nu >= kSlMidRows ? kSlMid : kSlSmall;
}

// Warp sums of the warp's NV per-lane values (the warp's slice or rows of
// tile jt of the item) in the working precision T, staged in shared memory
// wsum[(jt * 4 + a) * kWarps + warp].  Warps run through the item's tiles
// independently; the tile partials are formed once per item (item_finish).
template <int NV, typename T>
__device__ __forceinline__ void warp_part(T (&v)[NV], double* wsum, int jt) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    T x = v[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) wsum[(jt * 4 + a) * kWarps + wid] = (double)x;
  }
}

// After the tiles first .. first+nt-1 of a work item: tile partials (the
// warp sums of each tile added in warp order, FP64) into S.part; count the
// item; in the block that completed the system's last item (target items),
// thread 0 returns true with the totals over all of the system's tiles (in
// tile order, fixed tree).
template <int NV>
__device__ __forceinline__ bool item_finish(const BSys& S, const double* wsum, int64_t first, int nt, unsigned target,
                                            double (&tot)[NV]) {
  __shared__ double sh2[NV][kWarps];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if ((int)threadIdx.x < nt) {
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) s += wsum[(threadIdx.x * 4 + a) * kWarps + w];
      S.part[(first + threadIdx.x) * 4 + a] = s;
    }
    __threadfence();  // the tile partials before the count
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(S.ticket, 1u) == target - 1u;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // thread t adds tiles t, t + kBlk, ... in order; eight tiles' loads in flight
  double acc[NV];
#pragma unroll
  for (int a = 0; a < NV; ++a) acc[a] = 0.0;
  const double2* P = reinterpret_cast<const double2*>(S.part);
  int64_t b = threadIdx.x;
  for (; b + 7 * kBlk < S.ntiles; b += 8 * kBlk) {
    double2 lo[8], hi[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      lo[u] = __ldcg(P + (b + u * kBlk) * 2);
      if (NV > 2) hi[u] = __ldcg(P + (b + u * kBlk) * 2 + 1);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      acc[0] += lo[u].x;
      if (NV > 1) acc[NV > 1 ? 1 : 0] += lo[u].y;
      if (NV > 2) acc[NV > 2 ? 2 : 0] += hi[u].x;
      if (NV > 3) acc[NV > 3 ? 3 : 0] += hi[u].y;
    }
  }
  for (; b < S.ntiles; b += kBlk) {
    const double2 lo = __ldcg(P + b * 2);
    acc[0] += lo.x;
    if (NV > 1) acc[NV > 1 ? 1 : 0] += lo.y;
    if (NV > 2) {
      const double2 hi = __ldcg(P + b * 2 + 1);
      acc[NV > 2 ? 2 : 0] += hi.x;
      if (NV > 3) acc[NV > 3 ? 3 : 0] += hi.y;
    }
  }
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    double s = acc[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh2[a][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < kBlk / 32; ++w) s += sh2[a][w];
      tot[a] = s;
    }
    *S.ticket = 0u;
  }
  __syncthreads();
  return threadIdx.x == 0;
}

// ------------------------------------------------------------------ kernels
// With programmatic dependent launch (launch_pdl, pdl_wait) the kernels stage
// their first work item and its system descriptor before waiting on the
// previous kernel.

// Copy a system descriptor into shared memory (one 8-byte word per thread).
__device__ __forceinline__ void stage_sys(const BSys* __restrict__ src, BSys* dst) {
  static_assert(sizeof(BSys) % 8 == 0 && sizeof(BSys) / 8 <= kBlk, "descriptor staging");
  if (threadIdx.x < sizeof(BSys) / 8)
    reinterpret_cast<uint64_t*>(dst)[threadIdx.x] = __ldg(reinterpret_cast<const uint64_t*>(src) + threadIdx.x);
  __syncthreads();
}

// body(it, S) for each work item it = (slot, first tile, tiles) of this
// block, S its system's descriptor staged in shared memory.  The first
// item's descriptor is staged before the wait on the previous kernel (the
// item map and the descriptors are written before the graph runs).
template <typename F>
__device__ __forceinline__ void for_items(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                          const int* __restrict__ ntot, F&& body) {
  __shared__ BSys S;
  pdl_launch_dependents();
  const int total = *ntot;
  int t = blockIdx.x;
  int4 it = make_int4(0, 0, 0, 0);
  if (t < total) {
    it = items[t];
    stage_sys(sys + it.x, &S);
  }
  pdl_wait();
  while (t < total) {
    body(it, (const BSys&)S);
    t += gridDim.x;
    if (t >= total) break;
    const int prev = it.x;
    it = items[t];
    if (it.x != prev) {  // consecutive items of one system share the staged descriptor
      __syncthreads();   // every thread is done with the previous descriptor
      stage_sys(sys + it.x, &S);
    }
  }
}

// spmv slot: CG step length, or the FP64 residual of a replacement.
// COH: inside the persistent kernel, whose other blocks write p and x64
// between the phases (gathers through L2, not the read-only path).
template <bool IR, bool COH>
__device__ __forceinline__ void phase_spmv(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                           const int* __restrict__ nitems_total) {
  __shared__ double wsum[kItemMax * 4 * kWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for_items(sys, items, nitems_total, [&](const int4& it, const BSys& S) {
    const int mode = S.st[I_MODE];
    if (IR && (mode == M_CG || mode == M_STARTED)) {
      {
        for (int64_t j = it.y; j < it.y + it.z; ++j) {
          float pq = 0.f, rp = 0.f;
          for (int u = 0; u < S.sl; ++u) {
            const int64_t s = (j * S.sl + u) * kWarps + wid;
            const int64_t row = s * 32 + lane;
            if (s < S.A.nslices) {
              const bool in = row < S.A.nrows;
              const float xi = in ? S.p32[row] : 0.f;
              const float acc = S.A.d16 ? sell_row_acc<float, true, true, COH>(S.A, S.v32, S.p32, s, lane, xi)
                                        : sell_row_acc<float, false, true, COH>(S.A, S.v32, S.p32, s, lane, xi);
              if (in) {
                S.q32[row] = acc;
                pq += acc * xi;
                rp += S.r32[row] * xi;
              }
            }
          }
          float v[2] = {pq, rp};
          warp_part<2>(v, wsum, (int)(j - it.y));
        }
        double tot[2];
        if (item_finish<2>(S, wsum, it.y, it.z, (unsigned)*S.nitems, tot)) {
          S.sc[B_PQ] = tot[0];
          S.sc[B_ALPHA] = (tot[0] > 0.0 && isfinite(tot[0])) ? tot[1] / tot[0] : 0.0;
          if (mode == M_STARTED) S.st[I_MODE] = M_CG;
        }
      }
    } else if (mode == M_FOLD) {
      // FP64 residual check (both methods): FP32 refinement replacement, or
      // the FP64 recurrence's claim of convergence
      {
        for (int64_t j = it.y; j < it.y + it.z; ++j) {
          double rr = 0.0;
          for (int u = 0; u < S.sl; ++u) {
            const int64_t s = (j * S.sl + u) * kWarps + wid;
            const int64_t row = s * 32 + lane;
            if (s < S.A.nslices) {
              const double acc = S.A.d16 ? sell_row_resid<true, COH>(S.A, S.v64, S.x64, s, lane)
                                         : sell_row_resid<false, COH>(S.A, S.v64, S.x64, s, lane);
              if (row < S.A.nrows) {
                const double rv = S.b64[row] - acc;
                S.r64[row] = rv;
                rr += rv * rv;
              }
            }
          }
          double v[1] = {rr};
          warp_part<1>(v, wsum, (int)(j - it.y));
        }
        double tot[1];
        if (item_finish<1>(S, wsum, it.y, it.z, (unsigned)*S.nitems, tot)) {
          const double rrt = tot[0];
          S.sc[B_RRT] = rrt;
          S.st[I_REPL] += 1;
          const bool exact = !(rrt > 0.0) && isfinite(rrt);
          const bool conv = exact || rrt <= S.sc[B_TOL2] * S.sc[B_BN2];
          if (conv || !isfinite(rrt) || S.st[I_ITER] >= S.st[I_MAXIT] || (!IR && S.st[I_REPL] > 50)) {
            S.st[I_CONV] = conv ? 1 : 0;
            S.st[I_MODE] = M_DONE;
          } else {
            // FP32 refinement: keep the search direction unless the
            // recurrence broke down or its residual drifted far below the
            // true one; FP64: restart from the true residual
            const double rrec = S.sc[B_RREC];
            S.st[I_RESTART] = (!IR || S.st[I_BRK] || !(rrec > 0.0) || !(rrec >= 1e-6 * rrt)) ? 1 : 0;
            S.st[I_BRK] = 0;
            S.st[I_MODE] = M_RESTART;
          }
        }
      }
    } else if (!IR && (mode == M_CG || mode == M_STARTED)) {
      for (int64_t j = it.y; j < it.y + it.z; ++j) {
        double pq = 0.0;
        for (int u = 0; u < S.sl; ++u) {
          const int64_t s = (j * S.sl + u) * kWarps + wid;
          const int64_t row = s * 32 + lane;
          if (s < S.A.nslices) {
            const double acc = S.A.d16 ? sell_row_acc<double, true, false, COH>(S.A, S.v64, S.p64, s, lane, 0.0)
                                       : sell_row_acc<double, false, false, COH>(S.A, S.v64, S.p64, s, lane, 0.0);
            if (row < S.A.nrows) {
              S.q64[row] = acc;
              pq += acc * S.p64[row];
            }
          }
        }
        double v[1] = {pq};
        warp_part<1>(v, wsum, (int)(j - it.y));
      }
      double tot[1];
      if (item_finish<1>(S, wsum, it.y, it.z, (unsigned)*S.nitems, tot)) {
        S.sc[B_PQ] = tot[0];
        S.sc[B_ALPHA] = (tot[0] > 0.0 && isfinite(tot[0])) ? S.sc[B_RZ] / tot[0] : 0.0;
        if (mode == M_STARTED) S.st[I_MODE] = M_CG;
      }
    }
  });
}

template <bool IR>
__global__ void __launch_bounds__(kBlk, 5) b_spmv_k(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                                 const int* __restrict__ nitems_total) {
  phase_spmv<IR, false>(sys, items, nitems_total);
}

// update slot: x, r, z and beta; or the restart after a replacement.
template <bool IR>
__device__ __forceinline__ void phase_update(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                             const int* __restrict__ nitems_total) {
  __shared__ double wsum[kItemMax * 4 * kWarps];
  for_items(sys, items, nitems_total, [&](const int4& it, const BSys& S) {
    const int mode = S.st[I_MODE];
    if (IR) {
      if (mode == M_CG) {
        const double pq = S.sc[B_PQ];
        const bool brk = !(pq > 0.0) || !isfinite(pq);
        const float alpha = brk ? 0.f : (float)S.sc[B_ALPHA];
        for (int64_t j = it.y; j < it.y + it.z; ++j) {
          float prz = 0.f, prr = 0.f, pzo = 0.f;
#pragma unroll
          for (int u = 0; u < S.sl; ++u) {
            const int64_t row = (j * S.sl + u) * kBlk + threadIdx.x;
            if (row < S.A.nrows) {
              const float pi = S.p32[row];
              S.x32[row] += alpha * pi;
              const float ro = S.r32[row];
              const float ri = ro - alpha * S.q32[row];
              S.r32[row] = ri;
              const float zi = S.dinv32[row] * ri;
              S.z32[row] = zi;
              prz += ri * zi;
              prr += ri * ri;
              pzo += zi * ro;
            }
          }
          float v[3] = {prz, prr, pzo};
          warp_part<3>(v, wsum, (int)(j - it.y));
        }
        double tot[3];
        if (item_finish<3>(S, wsum, it.y, it.z, (unsigned)*S.nitems, tot)) {
          const double rz = tot[0], rr = tot[1];
          S.sc[B_BETA] = (rz - tot[2]) / S.sc[B_RZ];
          S.sc[B_RZ] = rz;
          S.sc[B_RR] = rr;
          const int itn = ++S.st[I_ITER];
          // the recurrence works on r / s with s = ||b||: converged at rtol^2
          const bool conv = rr <= S.sc[B_TOL2];
          const bool bad = brk || !isfinite(rz) || !isfinite(rr);
          bool ru;
          if (bad) {
            S.st[I_BRK] = 1;
            ru = true;
          } else {
            const double rn = sqrt(rr);
            if (rn > S.sc[B_RMAX]) S.sc[B_RMAX] = rn;
            if (conv) S.st[I_BRK] = 2;  // spent directions: restart from p = z
            ru = conv || itn >= S.st[I_MAXIT] || rn < S.sc[B_DELTA] * S.sc[B_RMAX];
          }
          if (ru) {
            const double sc2 = S.sc[B_SCALE] * S.sc[B_SCALE];
            S.sc[B_RREC] = rr * sc2;
            S.st[I_MODE] = M_FOLD;
          }
        }
      } else if (mode == M_RESTART) {
        const double inv = 1.0 / S.sc[B_SCALE];
        const int restart = S.st[I_RESTART];
        for (int64_t j = it.y; j < it.y + it.z; ++j) {
          float prz = 0.f;
#pragma unroll
          for (int u = 0; u < S.sl; ++u) {
            const int64_t row = (j * S.sl + u) * kBlk + threadIdx.x;
            if (row < S.A.nrows) {
              const float ri = (float)(S.r64[row] * inv);
              S.r32[row] = ri;
              const float zi = S.dinv32[row] * ri;
              S.z32[row] = zi;
              if (restart) S.p32[row] = zi;
              prz += ri * zi;
            }
          }
          float v[1] = {prz};
          warp_part<1>(v, wsum, (int)(j - it.y));
        }
        double tot[1];
        if (item_finish<1>(S, wsum, it.y, it.z, (unsigned)*S.nitems, tot)) {
          S.sc[B_RZ] = tot[0];
          S.sc[B_RMAX] = sqrt(S.sc[B_RRT]) / S.sc[B_SCALE];
          S.st[I_MODE] = M_STARTED;
        }
      }
    } else if (mode == M_CG) {
      const double pq = S.sc[B_PQ];
      const bool brk = !(pq > 0.0) || !isfinite(pq);
      const double alpha = brk ? 0.0 : S.sc[B_ALPHA];
      for (int64_t j = it.y; j < it.y + it.z; ++j) {
        double prz = 0.0, prr = 0.0;
#pragma unroll
        for (int u = 0; u < S.sl; ++u) {
          const int64_t row = (j * S.sl + u) * kBlk + threadIdx.x;
          if (row < S.A.nrows) {
            S.x64[row] += alpha * S.p64[row];
            const double ri = S.r64[row] - alpha * S.q64[row];
            S.r64[row] = ri;
            const double zi = S.dinv64[row] * ri;
            S.z64[row] = zi;
            prz += ri * zi;
            prr += ri * ri;
          }
        }
        double v[2] = {prz, prr};
        warp_part<2>(v, wsum, (int)(j - it.y));
      }
      double tot[2];
      if (item_finish<2>(S, wsum, it.y, it.z, (unsigned)*S.nitems, tot)) {
        const double rz = tot[0], rr = tot[1];
        S.sc[B_BETA] = rz / S.sc[B_RZ];
        S.sc[B_RZ] = rz;
        S.sc[B_RR] = rr;
        const int itn = ++S.st[I_ITER];
        const bool conv = rr <= S.sc[B_TOL2] * S.sc[B_BN2];
        const bool bad = brk || !isfinite(rz) || !isfinite(rr);
        if (conv && !bad && itn < S.st[I_MAXIT]) {
          S.st[I_MODE] = M_FOLD;  // the recurrence says converged: check the true residual
        } else if (conv || bad || itn >= S.st[I_MAXIT]) {
          S.st[I_CONV] = (conv && !bad) ? 1 : 0;
          S.st[I_MODE] = M_DONE;
        }
      }
    } else if (mode == M_RESTART) {
      // restart from the true residual: z = D r, p = z
      for (int64_t j = it.y; j < it.y + it.z; ++j) {
        double prz = 0.0;
#pragma unroll
        for (int u = 0; u < S.sl; ++u) {
          const int64_t row = (j * S.sl + u) * kBlk + threadIdx.x;
          if (row < S.A.nrows) {
            const double zi = S.dinv64[row] * S.r64[row];
            S.z64[row] = zi;
            S.p64[row] = zi;
            prz += S.r64[row] * zi;
          }
        }
        double v[1] = {prz};
        warp_part<1>(v, wsum, (int)(j - it.y));
      }
      double tot[1];
      if (item_finish<1>(S, wsum, it.y, it.z, (unsigned)*S.nitems, tot)) {
        S.sc[B_RZ] = tot[0];
        S.st[I_MODE] = M_STARTED;
      }
    }
  });
}

template <bool IR>
__global__ void __launch_bounds__(kBlk) b_update_k(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                                   const int* __restrict__ nitems_total) {
  phase_update<IR>(sys, items, nitems_total);
}

// p slot: p = z + beta p; in M_FOLD also x64 += s x32, x32 = 0.
template <bool IR>
__device__ __forceinline__ void phase_p(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                        const int* __restrict__ nitems_total) {
  for_items(sys, items, nitems_total, [&](const int4& it, const BSys& S) {
    const int mode = S.st[I_MODE];
    if (IR) {
      if (mode != M_CG && mode != M_FOLD) return;
      const float beta = (float)S.sc[B_BETA];
      const double s = S.sc[B_SCALE];
      for (int64_t row = (int64_t)it.y * S.sl * kBlk + threadIdx.x;
           row < (int64_t)(it.y + it.z) * S.sl * kBlk && row < S.A.nrows; row += kBlk) {
        S.p32[row] = S.z32[row] + beta * S.p32[row];
        if (mode == M_FOLD) {
          S.x64[row] += s * (double)S.x32[row];
          S.x32[row] = 0.f;
        }
      }
    } else if (mode == M_CG) {
      const double beta = S.sc[B_BETA];
      for (int64_t row = (int64_t)it.y * S.sl * kBlk + threadIdx.x;
           row < (int64_t)(it.y + it.z) * S.sl * kBlk && row < S.A.nrows; row += kBlk)
        S.p64[row] = S.z64[row] + beta * S.p64[row];
    }
  });
}

template <bool IR>
__global__ void __launch_bounds__(kBlk) b_p_k(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                              const int* __restrict__ nitems_total) {
  phase_p<IR>(sys, items, nitems_total);
}

// ------------------------------------------------------------------ persistent form
// (ELFEL_BATCH_PERSIST=1) One cooperative launch runs `iters` iterations of
// every active system: the three phases of an iteration in sequence,
// separated by a grid barrier; the arithmetic is that of the three kernels,
// so the iterates are the same bits.
// The barrier is a counter and a generation word; a block that waits longer
// than kBarSpins polls (about a second) records the timeout in err and
// every block leaves the kernel (err also stops the waiting of the others).
// The host reads err after the launch and fails the step.
struct GridBar {
  unsigned* count;
  unsigned* gen;
  int* err;
};
constexpr unsigned kBarSpins = 1u << 24;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ bool grid_sync(const GridBar& gb) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned g = ld_acquire_u32(gb.gen);
    __threadfence();  // this block's writes before its arrival
    if (atomicAdd(gb.count, 1u) == gridDim.x - 1u) {
      atomicExch(gb.count, 0u);
      __threadfence();
      atomicAdd(gb.gen, 1u);
    } else {
      unsigned spins = 0;
      while (ld_acquire_u32(gb.gen) == g) {
        if (*(volatile int*)gb.err) break;
        if (++spins > kBarSpins) {
          atomicExch(gb.err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();  // the other blocks' writes before ours reads
    ok = *(volatile int*)gb.err == 0;
  }
  __syncthreads();
  return ok != 0;
}

template <bool IR>
__global__ void __launch_bounds__(kBlk) b_persist_k(const BSys* __restrict__ sys, const int4* __restrict__ items,
                                                    const int* __restrict__ nitems_total, int iters, GridBar gb) {
  for (int k = 0; k < iters; ++k) {
    phase_spmv<IR, true>(sys, items, nitems_total);
    if (!grid_sync(gb)) return;
    phase_update<IR>(sys, items, nitems_total);
    if (!grid_sync(gb)) return;
    phase_p<IR>(sys, items, nitems_total);
    if (!grid_sync(gb)) return;
  }
}

// Start of one system (its own launch, before it joins the item map): x = 0,
// r = b (scaled by s = ||b|| for the FP32 recurrence), z = D r, p = z, r.z.
// Each tile is its own work item here.
template <bool IR>
__global__ void __launch_bounds__(kBlk) b_init_k(const BSys* __restrict__ sysp, const double* __restrict__ bn2p) {
  __shared__ double wsum[4 * kWarps];
  const BSys& S = *sysp;
  const double bn2 = *bn2p;
  for (int64_t j = blockIdx.x; j < S.ntiles; j += gridDim.x) {
    if (IR) {
      const double inv = bn2 > 0.0 ? 1.0 / sqrt(bn2) : 0.0;
      float prz = 0.f;
      for (int u = 0; u < S.sl; ++u) {
        const int64_t row = (j * S.sl + u) * kBlk + threadIdx.x;
        if (row < S.A.nrows) {
          S.x64[row] = 0.0;
          S.x32[row] = 0.f;
          const float ri = (float)(S.b64[row] * inv);
          S.r32[row] = ri;
          const float zi = S.dinv32[row] * ri;
          S.z32[row] = zi;
          S.p32[row] = zi;
          prz += ri * zi;
        }
      }
      float v[1] = {prz};
      warp_part<1>(v, wsum, 0);
    } else {
      double prz = 0.0;
      for (int u = 0; u < S.sl; ++u) {
        const int64_t row = (j * S.sl + u) * kBlk + threadIdx.x;
        if (row < S.A.nrows) {
          S.x64[row] = 0.0;
          const double ri = S.b64[row];
          S.r64[row] = ri;
          const double zi = S.dinv64[row] * ri;
          S.z64[row] = zi;
          S.p64[row] = zi;
          prz += ri * zi;
        }
      }
      double v[1] = {prz};
      warp_part<1>(v, wsum, 0);
    }
    double tot[1];
    if (item_finish<1>(S, wsum, j, 1, (unsigned)S.ntiles, tot)) {
      S.sc[B_RZ] = tot[0];
      S.sc[B_BN2] = bn2;
      S.sc[B_SCALE] = bn2 > 0.0 ? sqrt(bn2) : 1.0;
      S.sc[B_RMAX] = 1.0;
      S.st[I_CONV] = bn2 > 0.0 ? 0 : 1;
      S.st[I_MODE] = bn2 > 0.0 ? M_CG : M_DONE;
    }
  }
}

// Item map: active system k owns items off[k] .. off[k+1]-1, each of up to
// item_tiles consecutive tiles; item t = (slot, first tile, tiles).
__global__ void b_map_k(const int* __restrict__ off, const int* __restrict__ slot, const int* __restrict__ ntl,
                        int nact, int item_tiles, int4* __restrict__ items, int* __restrict__ ntot,
                        int* __restrict__ nitems) {
  const int total = off[nact];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid == 0) *ntot = total;
  if (tid < nact) nitems[slot[tid]] = off[tid + 1] - off[tid];
  for (int t = tid; t < total; t += gridDim.x * blockDim.x) {
    int lo = 0, hi = nact - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int t0 = (t - off[lo]) * item_tiles;
    items[t] = make_int4(slot[lo], t0, min(item_tiles, ntl[lo] - t0), 0);
  }
}

}  // namespace elfel

using namespace elfel;

namespace {

struct Slot {
  elfel_sysmat* m = nullptr;
  int state = 0;  // 0 free, 1 active, 2 done (result not taken)
  int64_t nu = 0, ntiles = 0;
  double rtol = 0.0;
  DBuf<double> part;
  std::chrono::steady_clock::time_point t_add, t_done;
};

// grid of one configuration: blocks per SM of the spmv and of the vector kernels
struct GridCfg {
  int spmv, vec;
};

}  // namespace

struct elfel_batch {
  elfel_ctx* h = nullptr;
  int method = ELFEL_PCG32_IR;
  int cap = 0;
  int iters = kGraphIters;
  std::vector<Slot> slots;
  DBuf<BSys> sys;
  DBuf<double> sc;
  DBuf<int> st;
  DBuf<unsigned> tickets;
  DBuf<int> nitems;  // work items per slot in the current map
  DBuf<int4> items;
  int64_t items_cap = 0;
  DBuf<int> ntot;
  DBuf<int> act;  // off[cap + 1], slot[cap], ntiles[cap]
  int64_t total_tiles = 0, total_items = 0;
  bool map_dirty = false;
  std::vector<int> hst;
  std::vector<int> done;
  // captured graphs per grid configuration, valid for the current item-map buffer
  std::vector<GridCfg> cfgs;
  std::vector<cudaGraphExec_t> graphs;
  int occ_spmv = 1, occ_vec = 1;
  // the persistent form (b_persist_k): its resident blocks per SM and the
  // grid barrier's words (count, generation, error)
  int persist = 0, occ_persist = 1;
  DBuf<unsigned> gbar;
  std::map<int, int> tuned;  // log2(tiles) bucket -> chosen configuration
  int64_t launches = 0, kernel_launches = 0;
};

namespace {

Ctx* ctx_of(elfel_batch* b) { return &b->h->c; }

void drop_graphs(elfel_batch* b) {
  for (cudaGraphExec_t& g : b->graphs)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

template <bool IR>
void launch_iteration(cudaStream_t s, elfel_batch* b, const GridCfg& g, int sms) {
  const unsigned g1 = (unsigned)(sms * g.spmv), g2 = (unsigned)(sms * g.vec);
  const BSys* sy = b->sys.p;
  const int4* it = b->items.p;
  const int* nt = b->ntot.p;
  launch_pdl(b_spmv_k<IR>, g1, kBlk, s, sy, it, nt);
  launch_pdl(b_update_k<IR>, g2, kBlk, s, sy, it, nt);
  launch_pdl(b_p_k<IR>, g2, kBlk, s, sy, it, nt);
}

int graph_for(elfel_batch* b, int k, cudaGraphExec_t* out) {
  Ctx* c = ctx_of(b);
  if (!b->graphs[k]) {
    cudaGraph_t g;
    ELFEL_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < b->iters; ++i) {
      if (b->method == ELFEL_PCG32_IR) launch_iteration<true>(c->stream, b, b->cfgs[k], c->sm_count);
      else launch_iteration<false>(c->stream, b, b->cfgs[k], c->sm_count);
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return fail(c, ELFEL_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graphs[k], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(c, ELFEL_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
  }
  *out = b->graphs[k];
  return ELFEL_OK;
}

// Rebuild the device item map from the active slots (in slot order).  Items
// hold item_tiles tiles, sized so that the map has about two items per
// resident block: few completion counts per system, balanced blocks.
int rebuild_map(elfel_batch* b) {
  Ctx* c = ctx_of(b);
  std::vector<int> sl, ntl;
  int64_t tiles = 0;
  for (int i = 0; i < b->cap; ++i)
    if (b->slots[i].state == 1) {
      sl.push_back(i);
      ntl.push_back((int)b->slots[i].ntiles);
      tiles += b->slots[i].ntiles;
    }
  const int nact = (int)sl.size();
  const int64_t target = 2LL * c->sm_count * std::max(b->occ_spmv, b->occ_vec);
  const int item_tiles = (int)std::min<int64_t>(kItemMax, std::max<int64_t>(1, tiles / std::max<int64_t>(target, 1)));
  std::vector<int> h(3 * (size_t)b->cap + 1, 0);
  int64_t nit = 0;
  for (int k = 0; k < nact; ++k) {
    h[k] = (int)nit;
    nit += (ntl[k] + item_tiles - 1) / item_tiles;
    h[b->cap + 1 + k] = sl[k];
    h[2 * b->cap + 1 + k] = ntl[k];
  }
  h[nact] = (int)nit;
  b->total_tiles = tiles;
  b->total_items = nit;
  if (nit > b->items_cap) {
    int64_t cap = std::max<int64_t>(b->items_cap * 2, 1024);
    while (cap < nit) cap *= 2;
    b->items.release(c);
    ELFEL_TRY(b->items.alloc(c, (size_t)cap));
    b->items_cap = cap;
    drop_graphs(b);  // graphs hold the old buffer
  }
  ELFEL_CUDA(c, cudaMemcpyAsync(b->act.p, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, c->stream));
  b_map_k<<<grid_for(std::max<int64_t>(std::max<int64_t>(nit, nact), 1), 256, (int64_t)c->sm_count * 8), 256, 0,
            c->stream>>>(b->act.p, b->act.p + b->cap + 1, b->act.p + 2 * b->cap + 1, nact, item_tiles, b->items.p,
                         b->ntot.p, b->nitems.p);
  ELFEL_LAUNCH_CHECK(c);
  b->map_dirty = false;
  return ELFEL_OK;
}

int read_states(elfel_batch* b) {
  Ctx* c = ctx_of(b);
  ELFEL_CUDA(c, cudaMemcpyAsync(b->hst.data(), b->st.p, sizeof(int) * b->hst.size(), cudaMemcpyDeviceToHost,
                                c->stream));
  unsigned bar[3] = {0, 0, 0};
  if (b->persist) ELFEL_CUDA(c, cudaMemcpyAsync(bar, b->gbar.p, sizeof(bar), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  if (bar[2]) return fail(c, ELFEL_ERR_CUDA, "batch: a grid barrier of the persistent iteration kernel timed out");
  const auto now = std::chrono::steady_clock::now();
  for (int i = 0; i < b->cap; ++i) {
    Slot& s = b->slots[i];
    if (s.state == 1 && b->hst[(size_t)i * I_COUNT + I_MODE] == M_DONE) {
      s.state = 2;
      s.t_done = now;
      b->done.push_back(i);
      b->map_dirty = true;
    }
  }
  return ELFEL_OK;
}

void tune_key(const elfel_batch* b, int bucket, char* key, size_t cap) {
  snprintf(key, cap, "batch_%s_tiles_2^%d", b->method == ELFEL_PCG32_IR ? "pcg32_ir" : "pcg64", bucket);
}

// Time each grid configuration on the live batch (each run is a graph of real
// iterations) and keep the fastest for this size bucket.
int autotune(elfel_batch* b, int bucket) {
  Ctx* c = ctx_of(b);
  const int n = (int)b->cfgs.size();
  std::vector<double> ms(n, 0.0);
  cudaEvent_t e0, e1;
  ELFEL_CUDA(c, cudaEventCreate(&e0));
  ELFEL_CUDA(c, cudaEventCreate(&e1));
  for (int k = 0; k < n; ++k) {
    cudaGraphExec_t g;
    ELFEL_TRY(graph_for(b, k, &g));
    ELFEL_CUDA(c, cudaEventRecord(e0, c->stream));
    ELFEL_CUDA(c, cudaGraphLaunch(g, c->stream));
    ELFEL_CUDA(c, cudaEventRecord(e1, c->stream));
    ELFEL_CUDA(c, cudaEventSynchronize(e1));
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    ms[k] = t;
    b->launches++;
    b->kernel_launches += 3LL * b->iters;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int best = 0;
  for (int k = 1; k < n; ++k)
    if (ms[k] < ms[best]) best = k;
  b->tuned[bucket] = best;
  char key[96];
  tune_key(b, bucket, key, sizeof(key));
  std::string cand;
  for (int k = 0; k < n; ++k) {
    char one[48];
    snprintf(one, sizeof(one), "%s%dx%d", k ? "," : "", b->cfgs[k].spmv, b->cfgs[k].vec);
    cand += one;
  }
  tune_record(c, key, cand, best, ms);
  return ELFEL_OK;
}

int bucket_of(int64_t tiles) {
  int k = 0;
  while ((1LL << (k + 1)) <= tiles) ++k;
  return k;
}

}  // namespace

// ------------------------------------------------------------------ internal API
namespace elfel {

int batch_add_dev(elfel_batch* b, elfel_sysmat* m, const double* F, const double* T, int t_dev, int64_t nu,
                  double rtol, int32_t maxit, int32_t* slot_out) {
  Ctx* c = ctx_of(b);
  if (!m || !m->h || m->h != b->h) return fail(c, ELFEL_ERR_ARG, "batch_add: system of another context");
  if (!m->finished) return fail(c, ELFEL_ERR_STATE, "batch_add: finish! the matrix first");
  if (m->nrow != m->ncol) return fail(c, ELFEL_ERR_ARG, "batch_add: K must be square");
  if (m->busy) return fail(c, ELFEL_ERR_STATE, "batch_add: the system is already in a batch");
  if (nu < 0 || nu > m->nrow || !T) return fail(c, ELFEL_ERR_ARG, "batch_add: nu outside 0..%lld", (long long)m->nrow);
  if (!F && !m->has_rhs) return fail(c, ELFEL_ERR_ARG, "batch_add: no right-hand side");
  if (!(rtol > 0.0) || maxit < 1) return fail(c, ELFEL_ERR_ARG, "batch_add: rtol > 0 and maxit >= 1 required");
  if (nu > (int64_t)0x7fffffff - kTileRowsMax) return fail(c, ELFEL_ERR_ARG, "batch_add: system too large");
  int k = -1;
  for (int i = 0; i < b->cap; ++i)
    if (b->slots[i].state == 0) {
      k = i;
      break;
    }
  if (k < 0) return fail(c, ELFEL_ERR_STATE, "batch_add: all %d slots in use", b->cap);
  cudaSetDevice(c->device);
  ELFEL_TRY(build_solver(m, nu));
  ELFEL_TRY(refresh_values(m, 0, b->method == ELFEL_PCG32_IR ? 1 : 0));
  SolverData* S = m->solver;
  Slot& s = b->slots[k];
  s.m = m;
  s.nu = nu;
  s.rtol = rtol;
  const int sl = tile_row_groups(nu);
  s.ntiles = (nu + (int64_t)sl * kBlk - 1) / ((int64_t)sl * kBlk);
  s.t_add = std::chrono::steady_clock::now();
  if (nu > 0) {
    ELFEL_TRY(lift_rhs(m, F, T, t_dev));
    ELFEL_TRY(s.part.alloc(c, (size_t)s.ntiles * 4));
  } else {
    ELFEL_CUDA(c, cudaMemcpyAsync(S->T64.p, T, sizeof(double) * m->nrow,
                                  t_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  }
  BSys d;
  memset(&d, 0, sizeof(d));
  d.A = S->view();
  d.v32 = S->A.v32.p;
  d.v64 = S->A.v64.p;
  d.dinv32 = S->dinv32.p;
  d.dinv64 = S->dinv64.p;
  d.x32 = S->xa32.p;
  d.r32 = S->r32.p;
  d.z32 = S->z32.p;
  d.p32 = S->p32.p;
  d.q32 = S->q32.p;
  d.x64 = S->x64.p;
  d.r64 = S->r64.p;
  d.z64 = S->z64.p;
  d.p64 = S->p64.p;
  d.q64 = S->q64.p;
  d.b64 = S->b64.p;
  d.ntiles = s.ntiles;
  d.sl = sl;
  d.part = s.part.p;
  d.ticket = b->tickets.p + k;
  d.nitems = b->nitems.p + k;
  d.sc = b->sc.p + (size_t)k * B_COUNT;
  d.st = b->st.p + (size_t)k * I_COUNT;
  double hsc[B_COUNT] = {0};
  int hst[I_COUNT] = {0};
  hsc[B_TOL2] = rtol * rtol;
  double delta = 0.1;  // residual-replacement threshold (tuning knob)
  if (const char* e = getenv("ELFEL_RU_DELTA")) {
    const double v = atof(e);
    if (v > 0.0 && v < 1.0) delta = v;
  }
  hsc[B_DELTA] = delta;
  hst[I_MAXIT] = maxit;
  hst[I_MODE] = nu > 0 ? M_IDLE : M_DONE;
  hst[I_CONV] = nu > 0 ? 0 : 1;
  ELFEL_CUDA(c, cudaMemcpyAsync(b->sys.p + k, &d, sizeof(d), cudaMemcpyHostToDevice, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(d.sc, hsc, sizeof(hsc), cudaMemcpyHostToDevice, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(d.st, hst, sizeof(hst), cudaMemcpyHostToDevice, c->stream));
  ELFEL_CUDA(c, cudaMemsetAsync(d.ticket, 0, sizeof(unsigned), c->stream));
  if (nu > 0) {
    const unsigned g = (unsigned)std::min<int64_t>(s.ntiles, (int64_t)c->sm_count * 8);
    if (b->method == ELFEL_PCG32_IR) b_init_k<true><<<g, kBlk, 0, c->stream>>>(b->sys.p + k, S->scal.p + S_BN2);
    else b_init_k<false><<<g, kBlk, 0, c->stream>>>(b->sys.p + k, S->scal.p + S_BN2);
    ELFEL_LAUNCH_CHECK(c);
    b->kernel_launches++;
    s.state = 1;
    b->map_dirty = true;
  } else {
    s.state = 2;
    s.t_done = s.t_add;
    b->done.push_back(k);
  }
  m->busy = 1;
  // copy the pageable host arrays before they go out of scope
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  *slot_out = k;
  return ELFEL_OK;
}

int batch_step(elfel_batch* b, int32_t graphs, int32_t* active) {
  Ctx* c = ctx_of(b);
  cudaSetDevice(c->device);
  if (b->map_dirty) ELFEL_TRY(rebuild_map(b));
  for (int gi = 0; b->persist && gi < graphs && b->total_tiles > 0; ++gi) {
    // one cooperative launch of iters iterations (all blocks resident)
    const BSys* sy = b->sys.p;
    const int4* itp = b->items.p;
    const int* ntp = b->ntot.p;
    int iters = b->iters;
    GridBar gb{b->gbar.p, b->gbar.p + 1, reinterpret_cast<int*>(b->gbar.p + 2)};
    void* args[] = {(void*)&sy, (void*)&itp, (void*)&ntp, (void*)&iters, (void*)&gb};
    const dim3 grid((unsigned)(c->sm_count * b->occ_persist)), block(kBlk);
    if (b->method == ELFEL_PCG32_IR)
      ELFEL_CUDA(c, cudaLaunchCooperativeKernel((const void*)b_persist_k<true>, grid, block, args, 0, c->stream));
    else
      ELFEL_CUDA(c, cudaLaunchCooperativeKernel((const void*)b_persist_k<false>, grid, block, args, 0, c->stream));
    b->launches++;
    b->kernel_launches++;
  }
  for (int gi = 0; !b->persist && gi < graphs && b->total_tiles > 0; ++gi) {
    const int bucket = bucket_of(b->total_tiles);
    auto it = b->tuned.find(bucket);
    if (it == b->tuned.end()) {
      char key[96];
      tune_key(b, bucket, key, sizeof(key));
      const int known = tune_lookup(c, key);  // tuned earlier in this context
      if (known < 0 && c->tune) {
        ELFEL_TRY(autotune(b, bucket));
        continue;  // the tuning runs were iterations of this step
      }
      b->tuned[bucket] = known < 0 ? 0 : known;
      it = b->tuned.find(bucket);
    }
    cudaGraphExec_t g;
    ELFEL_TRY(graph_for(b, it->second, &g));
    ELFEL_CUDA(c, cudaGraphLaunch(g, c->stream));
    b->launches++;
    b->kernel_launches += 3LL * b->iters;
  }
  ELFEL_TRY(read_states(b));
  if (b->map_dirty) ELFEL_TRY(rebuild_map(b));
  int n = 0;
  for (const Slot& s : b->slots) n += s.state == 1;
  if (active) *active = n;
  if (c->trace)
    fprintf(stderr, "[elfel batch] step: %d active, %lld tiles in %lld items, %zu finished waiting\n", n,
            (long long)b->total_tiles, (long long)b->total_items, b->done.size());
  return ELFEL_OK;
}

// Result of a finished slot: x (original order) into T_out[0:nu] and the data
// values into T_out[nu:n] (device or host memory), the final FP64 residual
// b - K_ff x in stats; frees the slot.
int batch_take(elfel_batch* b, int32_t k, double* T_out, int t_dev, elfel_solve_stats* stats) {
  Ctx* c = ctx_of(b);
  if (k < 0 || k >= b->cap || b->slots[k].state != 2)
    return fail(c, ELFEL_ERR_STATE, "batch_result: slot %d has no finished solve", k);
  cudaSetDevice(c->device);
  Slot& s = b->slots[k];
  elfel_sysmat* m = s.m;
  SolverData* S = m->solver;
  const int64_t n = m->nrow, nu = s.nu;
  const cudaMemcpyKind kind = t_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  int hst[I_COUNT] = {0};
  ELFEL_CUDA(c, cudaMemcpyAsync(hst, b->st.p + (size_t)k * I_COUNT, sizeof(hst), cudaMemcpyDeviceToHost, c->stream));
  double rr = 0.0, bn2 = 0.0;
  if (nu > 0) {
    ELFEL_TRY(solution_residual(m));
    ELFEL_CUDA(c, cudaMemcpyAsync(&rr, S->scal.p + S_RR, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaMemcpyAsync(&bn2, S->scal.p + S_BN2, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (T_out) ELFEL_CUDA(c, cudaMemcpyAsync(T_out, S->xo64.p, sizeof(double) * nu, kind, c->stream));
  }
  if (T_out && n > nu)
    ELFEL_CUDA(c, cudaMemcpyAsync(T_out + nu, S->T64.p + nu, sizeof(double) * (n - nu), kind, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  elfel_solve_stats st;
  memset(&st, 0, sizeof(st));
  st.iterations = hst[I_ITER];
  st.refinements = hst[I_REPL];
  st.relres = bn2 > 0.0 ? sqrt(rr / bn2) : 0.0;
  st.converged = (nu == 0 || st.relres <= s.rtol) ? 1 : 0;
  st.seconds = std::chrono::duration<double>(s.t_done - s.t_add).count();
  if (stats) *stats = st;
  s.part.release(c);
  s.state = 0;
  s.m = nullptr;
  m->busy = 0;
  b->done.erase(std::remove(b->done.begin(), b->done.end(), k), b->done.end());
  return ELFEL_OK;
}

int batch_counts(elfel_batch* b, int64_t* launches, int64_t* kernels) {
  *launches = b->launches;
  *kernels = b->kernel_launches;
  return ELFEL_OK;
}

}  // namespace elfel

// ------------------------------------------------------------------ C ABI
extern "C" int elfel_batch_create(elfel_ctx* h, int32_t method, int32_t capacity, elfel_batch** out) {
  if (!h || !out) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  if (method != ELFEL_PCG64 && method != ELFEL_PCG32_IR)
    return fail(c, ELFEL_ERR_UNSUPPORTED, "batch: methods ELFEL_PCG64 and ELFEL_PCG32_IR are batched");
  if (capacity < 1 || capacity > 65536) return fail(c, ELFEL_ERR_ARG, "batch: capacity 1..65536");
  cudaSetDevice(c->device);
  elfel_batch* b = new elfel_batch();
  b->h = h;
  b->method = method;
  b->cap = capacity;
  b->slots.resize(capacity);
  b->hst.assign((size_t)capacity * I_COUNT, 0);
  int rc = ELFEL_OK;
  if ((rc = b->sys.alloc(c, (size_t)capacity)) || (rc = b->sc.alloc(c, (size_t)capacity * B_COUNT)) ||
      (rc = b->st.alloc(c, (size_t)capacity * I_COUNT)) || (rc = b->tickets.alloc(c, (size_t)capacity)) ||
      (rc = b->nitems.alloc(c, (size_t)capacity)) || (rc = b->ntot.alloc(c, 1)) ||
      (rc = b->act.alloc(c, 3 * (size_t)capacity + 1))) {
    delete b;
    return rc;
  }
  cudaMemsetAsync(b->st.p, 0, sizeof(int) * capacity * I_COUNT, c->stream);
  cudaMemsetAsync(b->tickets.p, 0, sizeof(unsigned) * capacity, c->stream);
  cudaMemsetAsync(b->nitems.p, 0, sizeof(int) * capacity, c->stream);
  cudaMemsetAsync(b->ntot.p, 0, sizeof(int), c->stream);
  // resident blocks per SM of the kernels: the grid configurations tried
  int o1 = 1, o2 = 1;
  if (method == ELFEL_PCG32_IR) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, b_spmv_k<true>, kBlk, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, b_update_k<true>, kBlk, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, b_spmv_k<false>, kBlk, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, b_update_k<false>, kBlk, 0);
  }
  o1 = std::max(o1, 1);
  o2 = std::max(o2, 1);
  b->occ_spmv = o1;
  b->occ_vec = o2;
  // the persistent form when ELFEL_BATCH_PERSIST=1 (and the device can launch
  // it cooperatively).  Measured on GB300 it is slower than the graphs of
  // three kernels (its three grid barriers per iteration cost more than the
  // launches they replace, and one grid serves all phases), so the graphs
  // stay the default.
  int coop = 0, op = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device);
  if (method == ELFEL_PCG32_IR)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&op, b_persist_k<true>, kBlk, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&op, b_persist_k<false>, kBlk, 0);
  const char* pe = getenv("ELFEL_BATCH_PERSIST");
  b->persist = (coop && op > 0 && pe && pe[0] == '1') ? 1 : 0;
  b->occ_persist = std::max(op, 1);
  if (b->persist) {
    if ((rc = b->gbar.alloc(c, 4))) {
      delete b;
      return rc;
    }
    cudaMemsetAsync(b->gbar.p, 0, 4 * sizeof(unsigned), c->stream);
  }
  b->cfgs = {{o1, o2}, {std::max(o1 / 2, 1), std::max(o2 / 2, 1)}, {2 * o1, o2}, {o1, 2 * o2}};
  b->graphs.assign(b->cfgs.size(), nullptr);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    delete b;
    return fail(c, ELFEL_ERR_CUDA, "batch_create: %s", cudaGetErrorString(cudaGetLastError()));
  }
  *out = b;
  return ELFEL_OK;
}

extern "C" int elfel_batch_destroy(elfel_batch* b) {
  if (!b) return ELFEL_OK;
  Ctx* c = &b->h->c;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (Slot& s : b->slots) {
    s.part.release(c);
    if (s.m) s.m->busy = 0;
  }
  drop_graphs(b);
  b->gbar.release(c);
  b->sys.release(c);
  b->sc.release(c);
  b->st.release(c);
  b->tickets.release(c);
  b->nitems.release(c);
  b->items.release(c);
  b->ntot.release(c);
  b->act.release(c);
  delete b;
  return ELFEL_OK;
}

extern "C" int elfel_batch_add(elfel_batch* b, elfel_sysmat* m, const double* F, const double* T, int64_t nu,
                               double rtol, int32_t maxit, int32_t* slot) {
  if (!b || !slot) return ELFEL_ERR_ARG;
  return batch_add_dev(b, m, F, T, 0, nu, rtol, maxit, slot);
}

extern "C" int elfel_batch_step(elfel_batch* b, int32_t graphs, int32_t* active) {
  if (!b) return ELFEL_ERR_ARG;
  if (graphs < 1) return fail(&b->h->c, ELFEL_ERR_ARG, "batch_step: graphs >= 1");
  return batch_step(b, graphs, active);
}

extern "C" int elfel_batch_done(elfel_batch* b, int32_t* slots, int32_t cap, int32_t* n) {
  if (!b || !n || (cap > 0 && !slots)) return ELFEL_ERR_ARG;
  const int k = std::min<int>((int)b->done.size(), std::max(cap, 0));
  for (int i = 0; i < k; ++i) slots[i] = b->done[i];
  *n = (int32_t)b->done.size();
  return ELFEL_OK;
}

extern "C" int elfel_batch_result(elfel_batch* b, int32_t slot, double* T, elfel_solve_stats* stats) {
  if (!b) return ELFEL_ERR_ARG;
  return batch_take(b, slot, T, 0, stats);
}
