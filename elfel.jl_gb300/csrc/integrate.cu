// Element integration kernels: one thread per element, a CTA per batch of
// kIntThreads elements.
//   (a) the batch's connectivity is loaded into shared memory with coalesced
//       loads, node coordinates are gathered as 16-byte double2 loads;
//   (b) basis values / parametric gradients at the quadrature points are
//       staged once per CTA in shared memory;
//   (c) Jacobian, inverse, gradients and the element-matrix products run in
//       registers; results are staged in shared memory and written out as one
//       contiguous, coalesced record block per CTA.
// Element records are consumed by reduce_values() through the slot map.
//
// Weak forms restated from the reference (Elfel.jl v0.4.0):
//   heat        test/test_heat.jl:49-54
//   elasticity  test/test_elasticity.jl:150-167
//   Stokes TH   test/test_stokes.jl:645-652 (vector Laplacian form)
// Geometry: src/FElements.jl:148-168 (J = sum_j x_j (x) gradNpar_j, det J),
//           src/QPIterators.jl:132-140 (gradN = gradNpar / J).
//
// Straight-sided elements (T3 always; T6 when each midside node is exactly the
// midpoint of its edge) have a constant Jacobian.  For them the quadrature sum
// is reorganised with reference tensors precomputed from the same rule:
//   ke_ij = kappa*det * sum_q w_q gradN_i(q).gradN_j(q)
//         = c11*S11_ij + c22*S22_ij + c12*S12_ij,  S^{ab}_ij = sum_q w_q dN_i/dxi_a dN_j/dxi_b
// (the tensor representation of Kirby & Logg's FFC).  Curved T6 elements take
// the per-quadrature-point path, which mirrors the reference loop.
#include "integrate.cuh"
#include "floatpair.cuh"
#include "t6r.cuh"

namespace elfel {

// ------------------------------------------------------------------ tables
static void bfun_host(int nn, double r, double s, double* N, double* G) {
  if (nn == 3) {
    N[0] = 1.0 - r - s; N[1] = r; N[2] = s;
    G[0] = -1.0; G[1] = -1.0; G[2] = 1.0; G[3] = 0.0; G[4] = 0.0; G[5] = 1.0;
  } else {
    double t = 1.0 - r - s;
    N[0] = t * (t + t - 1); N[1] = r * (r + r - 1); N[2] = s * (s + s - 1);
    N[3] = 4 * r * t; N[4] = 4 * r * s; N[5] = 4 * s * t;
    G[0] = -3 + 4 * r + 4 * s; G[1] = -3 + 4 * r + 4 * s;
    G[2] = 4 * r - 1;          G[3] = 0.0;
    G[4] = 0.0;                G[5] = 4 * s - 1;
    G[6] = 4 - 8 * r - 4 * s;  G[7] = -4 * r;
    G[8] = 4 * s;              G[9] = 4 * r;
    G[10] = -4 * s;            G[11] = 4 - 4 * r - 8 * s;
  }
}

int make_tables(int nn, int npts, const double* pc, const double* w, QPTab* t) {
  if (npts < 1 || npts > kMaxQP || (nn != 3 && nn != 6)) return ELFEL_ERR_ARG;
  memset(t, 0, sizeof(*t));
  t->npts = npts;
  t->nn = nn;
  for (int q = 0; q < npts; ++q) {
    t->w[q] = w[q];
    double Np[3], Gp[6];
    bfun_host(nn, pc[2 * q], pc[2 * q + 1], t->N[q], &t->G[q][0][0]);
    bfun_host(3, pc[2 * q], pc[2 * q + 1], Np, Gp);
    for (int j = 0; j < 3; ++j) t->Np[q][j] = Np[j];
  }
  // reference tensors for straight-sided elements
  for (int i = 0; i < nn; ++i) {
    double P = 0.0;
    for (int q = 0; q < npts; ++q) P += t->w[q] * t->N[q][i];
    t->P[i] = P;
    for (int j = 0; j < nn; ++j) {
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
          double s = 0.0;
          for (int q = 0; q < npts; ++q) s += t->w[q] * t->G[q][i][a] * t->G[q][j][b];
          t->S[a][b][i * 6 + j] = s;
        }
    }
    for (int j = 0; j < 3; ++j)
      for (int a = 0; a < 2; ++a) {
        double s = 0.0;
        for (int q = 0; q < npts; ++q) s += t->w[q] * t->Np[q][j] * t->G[q][i][a];
        t->T[a][i * 3 + j] = s;
      }
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int q = 0; q < npts; ++q) s += t->w[q] * t->Np[q][j] * t->Np[q][j];
      t->Mp[j] = s;
    }
  }
  return ELFEL_OK;
}

// ------------------------------------------------------------------ helpers
template <int NN>
struct Geo {
  double x[NN], y[NN];
};

template <int NN>
__device__ __forceinline__ bool straight_sided(const Geo<NN>& g) {
  if (NN == 3) return true;
  return g.x[3] == 0.5 * (g.x[0] + g.x[1]) && g.y[3] == 0.5 * (g.y[0] + g.y[1]) &&
         g.x[4] == 0.5 * (g.x[1] + g.x[2]) && g.y[4] == 0.5 * (g.y[1] + g.y[2]) &&
         g.x[5] == 0.5 * (g.x[2] + g.x[0]) && g.y[5] == 0.5 * (g.y[2] + g.y[0]);
}

// Stage the element tables of a CTA in shared memory.
struct SmemTab {
  double w[kMaxQP];
  double N[kMaxQP][6];
  double G[kMaxQP][6][2];
  double Np[kMaxQP][3];
};

__device__ __forceinline__ void stage_tables(const QPTab& t, SmemTab* s) {
  for (int k = threadIdx.x; k < t.npts; k += blockDim.x) s->w[k] = t.w[k];
  for (int k = threadIdx.x; k < t.npts * 6; k += blockDim.x) (&s->N[0][0])[k] = (&t.N[0][0])[k];
  for (int k = threadIdx.x; k < t.npts * 12; k += blockDim.x) (&s->G[0][0][0])[k] = (&t.G[0][0][0])[k];
  for (int k = threadIdx.x; k < t.npts * 3; k += blockDim.x) (&s->Np[0][0])[k] = (&t.Np[0][0])[k];
}

// Load a CTA's connectivity tile (coalesced) and gather this thread's nodes.
template <int NN, int NT = kIntThreads>
__device__ __forceinline__ void load_geo(const int32_t* __restrict__ conn, const double2* __restrict__ xy, int64_t e0,
                                         int64_t nel, int32_t* sconn, Geo<NN>& g, int32_t* nodes) {
  const int64_t base = e0 * NN;
  const int64_t lim = nel * NN;
  for (int k = threadIdx.x; k < NT * NN; k += NT) {
    int64_t gi = base + k;
    sconn[k] = gi < lim ? __ldg(conn + gi) : 0;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    int32_t n = sconn[threadIdx.x * NN + j];
    if (nodes) nodes[j] = n;
    double2 p = __ldg(xy + n);
    g.x[j] = p.x;
    g.y[j] = p.y;
  }
}

// Write a CTA's records, staged as acc[k * (NT + 1) + t], to
// out[(e0 + t) * rec + k] in one contiguous pass.
template <int NT = kIntThreads>
__device__ __forceinline__ void write_records(const double* acc, int rec, int64_t e0, int64_t nel, double* out) {
  __syncthreads();
  const int64_t nvalid = min((int64_t)NT, nel - e0);
  const int64_t total = nvalid * rec;
  double* dst = out + e0 * rec;
  for (int64_t L = threadIdx.x; L < total; L += NT) {
    int t = (int)(L / rec), k = (int)(L - (int64_t)t * rec);
    dst[L] = acc[k * (NT + 1) + t];
  }
}

// Write entries k0 .. k0 + nk - 1 of a CTA's records, staged as
// acc[kk * (NT + 1) + t], to out[(e0 + t) * rec + k0 + kk].
template <int NT = kIntThreads>
__device__ __forceinline__ void write_records_part(const double* acc, int rec, int k0, int nk, int64_t e0,
                                                   int64_t nel, double* out) {
  __syncthreads();
  const int nvalid = (int)min((int64_t)NT, nel - e0);
  const int total = nvalid * nk;
  double* dst = out + e0 * rec + k0;
  for (int L = threadIdx.x; L < total; L += NT) {
    const int t = L / nk, kk = L - t * nk;
    dst[(int64_t)t * rec + kk] = acc[kk * (NT + 1) + t];
  }
}

// The same with compile-time widths: in a full CTA every thread writes NK
// values, its (element, entry) pair advancing by (NT / NK, NT % NK) per value
// (no division in the loop).
template <int NT, int REC, int NK>
__device__ __forceinline__ void write_records_fixed(const double* acc, int k0, int64_t e0, int64_t nel,
                                                    double* out) {
  if (e0 + NT > nel) {
    write_records_part<NT>(acc, REC, k0, NK, e0, nel, out);
    return;
  }
  __syncthreads();
  constexpr int DT = NT / NK, DK = NT % NK;
  double* dst = out + e0 * REC + k0;
  int t = (int)threadIdx.x / NK, kk = (int)threadIdx.x - t * NK;
#pragma unroll
  for (int i = 0; i < NK; ++i) {
    dst[t * REC + kk] = acc[kk * (NT + 1) + t];
    t += DT;
    kk += DK;
    if (kk >= NK) {
      kk -= NK;
      ++t;
    }
  }
}

// ------------------------------------------------------------------ heat
// Structural zeros of the T6 reference tensors for quadrature rules that
// integrate the products of the (linear) parametric gradients exactly, e.g.
// the 3-point rule: bit k = stored entry k (k = j(j+1)/2 + i, i <= j) has a
// nonzero coefficient in S11, S22, S12 + S21; bit j of kT6P = the element
// load vector entry j, sum_q w_q N_j, is nonzero (the vertex functions of P2
// integrate to zero).  With pattern kPatT6 the straight-sided branch skips
// the zero terms: 34 of 63 FP64 multiply-adds remain.
constexpr uint32_t kT6S11 = 0x1842c7u, kT6S22 = 0x12e229u, kT6S12 = 0x1efadbu, kT6P = 0x38u;
constexpr int kPatGeneric = 0, kPatT6 = 1, kPatT6R = 2;

// Rules that integrate the products of the parametric gradients exactly give
// the exact T6 tensors, whose stored entries (S11, S22, S12 + S21) are
// rational multiples of seven directions: with c11 = q11 s, c22 = q22 s,
// c12 = -q12 s (q11 = J22^2 + J12^2, q22 = J21^2 + J11^2, q12 = J22 J21 +
// J12 J11, s = kappa / det J) and u = q11 - q12, v = q22 - q12,
//   k0 = (u + v) s/2   k1 = u s/6   k2 = q11 s/2   k3 = v s/6   k4 = q12 s/6
//   k5 = q22 s/2       k6 = k7 = -u 2s/3   k19 = 2 k6   k15 = k17 = -v 2s/3
//   k13 = 2 k15        k11 = k12 = -q12 2s/3   k18 = 2 k11
//   k9 = k14 = k20 = 2 (u + q22) 2s/3        k8 = k10 = k16 = 0,
// and the element load is Q det / 6 at the midside nodes, 0 at the vertices.
// kPatT6R evaluates that form: 45 instead of 63 FP64 operations per element.
constexpr double kT6Exact[21][3] = {
    {0.5, 0.5, 1.0},      {1. / 6, 0, 1. / 6},  {0.5, 0, 0},          {0, 1. / 6, 1. / 6},   {0, 0, -1. / 6},
    {0, 0.5, 0},          {-2. / 3, 0, -2. / 3}, {-2. / 3, 0, -2. / 3}, {0, 0, 0},             {4. / 3, 4. / 3, 4. / 3},
    {0, 0, 0},            {0, 0, 2. / 3},        {0, 0, 2. / 3},        {0, -4. / 3, -4. / 3}, {4. / 3, 4. / 3, 4. / 3},
    {0, -2. / 3, -2. / 3}, {0, 0, 0},            {0, -2. / 3, -2. / 3}, {0, 0, 4. / 3},        {-4. / 3, 0, -4. / 3},
    {4. / 3, 4. / 3, 4. / 3}};

// Per-element flag: 1 when the element is straight-sided (the Jacobian is
// constant and the reference-tensor form applies).  Computed once per
// geometry, not per assembly.
template <int NN>
__global__ void straight_k(int64_t nel, const int32_t* __restrict__ conn, const double2* __restrict__ xy,
                           uint8_t* __restrict__ flag, unsigned long long* __restrict__ ncurved) {
  unsigned long long curved = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nel; e += (int64_t)gridDim.x * blockDim.x) {
    Geo<NN> g;
#pragma unroll
    for (int j = 0; j < NN; ++j) {
      const double2 p = xy[conn[e * NN + j]];
      g.x[j] = p.x;
      g.y[j] = p.y;
    }
    const bool s = straight_sided<NN>(g);
    flag[e] = s ? 1 : 0;
    curved += s ? 0 : 1;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) curved += __shfl_down_sync(0xffffffffu, curved, o);
  if ((threadIdx.x & 31) == 0 && curved) atomicAdd(ncurved, curved);
}

int launch_straight(Ctx* c, int nn, int64_t nel, const int32_t* conn, const double* xy, uint8_t* flag,
                    int64_t* ncurved) {
  *ncurved = 0;
  if (nel == 0) return ELFEL_OK;
  DBuf<unsigned long long> cnt;
  ELFEL_TRY(cnt.alloc(c, 1));
  ELFEL_CUDA(c, cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), c->stream));
  const unsigned grid = grid_for(nel, 256, (int64_t)c->sm_count * 16);
  if (nn == 3) straight_k<3><<<grid, 256, 0, c->stream>>>(nel, conn, (const double2*)xy, flag, cnt.p);
  else straight_k<6><<<grid, 256, 0, c->stream>>>(nel, conn, (const double2*)xy, flag, cnt.p);
  ELFEL_LAUNCH_CHECK(c);
  unsigned long long h = 0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  cnt.release(c);
  *ncurved = (int64_t)h;
  return ELFEL_OK;
}

// The T6 zero pattern of a table, when its tensors have exactly the zeros of
// kT6S11/kT6S22/kT6S12/kT6P (entries below 1e-13 of the largest count as
// zero: quadrature residues); else the generic pattern.
int heat_pattern(int nn, const QPTab& t) {
  if (nn != 6) return kPatGeneric;
  double mx = 0.0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int k = 0; k < 36; ++k) mx = fmax(mx, fabs(t.S[a][b][k]));
  const double tiny = 1e-13 * mx;
  uint32_t m11 = 0, m22 = 0, m12 = 0, mp = 0;
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i <= j; ++i) {
      const int k = j * (j + 1) / 2 + i;
      if (fabs(t.S[0][0][i * 6 + j]) > tiny) m11 |= 1u << k;
      if (fabs(t.S[1][1][i * 6 + j]) > tiny) m22 |= 1u << k;
      if (fabs(t.S[0][1][i * 6 + j] + t.S[1][0][i * 6 + j]) > tiny) m12 |= 1u << k;
    }
  double pmax = 0.0;
  for (int j = 0; j < 6; ++j) pmax = fmax(pmax, fabs(t.P[j]));
  for (int j = 0; j < 6; ++j)
    if (fabs(t.P[j]) > 1e-13 * pmax) mp |= 1u << j;
  if (!(m11 == kT6S11 && m22 == kT6S22 && m12 == kT6S12 && mp == kT6P)) return kPatGeneric;
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i <= j; ++i) {
      const double* x = kT6Exact[j * (j + 1) / 2 + i];
      if (fabs(t.S[0][0][i * 6 + j] - x[0]) > 1e-14 || fabs(t.S[1][1][i * 6 + j] - x[1]) > 1e-14 ||
          fabs(t.S[0][1][i * 6 + j] + t.S[1][0][i * 6 + j] - x[2]) > 1e-14)
        return kPatT6;
    }
  for (int j = 3; j < 6; ++j)
    if (fabs(t.P[j] - 1.0 / 6.0) > 1e-15) return kPatT6;
  return kPatT6R;
}

// The 8 bases in FP64: the fallback of t6r_bases_pair for elements outside
// its accuracy range.
__device__ __forceinline__ void t6r_bases_fp64(double J11, double J12, double J21, double J22, double kap, double Q,
                                               double P6, double* b) {
  const double det = __fma_rn(J11, J22, -__dmul_rn(J21, J12));
  const double s = __ddiv_rn(kap, det);
  const double q11 = __fma_rn(J22, J22, __dmul_rn(J12, J12));
  const double q22 = __fma_rn(J21, J21, __dmul_rn(J11, J11));
  const double q12 = __fma_rn(J22, J21, __dmul_rn(J12, J11));
  const double u = __dsub_rn(q11, q12), v = __dsub_rn(q22, q12);
  const double s2 = __dmul_rn(s, 0.5), s6 = __dmul_rn(s, 1.0 / 6.0);
  b[0] = __dmul_rn(__dadd_rn(u, v), s2);
  b[1] = __dmul_rn(u, s6);
  b[2] = __dmul_rn(q11, s2);
  b[3] = __dmul_rn(v, s6);
  b[4] = __dmul_rn(q12, s6);
  b[5] = __dmul_rn(q22, s2);
  b[6] = __dmul_rn(__dmul_rn(__dadd_rn(u, q22), s6), 8.0);
  b[7] = __dmul_rn(__dmul_rn(Q, det), P6);
}

// The 8 bases in float pairs (48-bit significands; see floatpair.cuh): J is
// scaled by 2^-k so that max |J'| is in [1, 2), kappa and Q to [1, 2) by their
// own powers of two, and the powers come back in the exponents of the
// results.  Only the 4 coordinate differences (in the caller) and 8 joins to
// double are FP64 instructions (about 30 in t6r_bases_fp64).  Elements with
// det J' < 1/4 (strongly distorted: the pair subtraction in det J' would cost
// more than 2^-42 relative accuracy) return false and take the FP64 form.
__device__ __forceinline__ bool t6r_bases_pair(double J11, double J12, double J21, double J22, double kap, double Q,
                                               double P6, double* bs) {
  const int em = max(max(dexp(J11), dexp(J12)), max(dexp(J21), dexp(J22)));
  const int k = em - 1023;
  const int kk = dexp(kap) - 1023, kq = dexp(Q) == 0 ? 0 : dexp(Q) - 1023;  // Q = 0: no scaling needed
  if (em == 0 || k < -400 || k > 400 || kk < -900 || kk > 900 || kq + 2 * k < -900 || kq + 2 * k > 900) return false;
  f2 A, B, C, D, kp, qp, p6, sixth;
  bool ok = split_scaled(J11, k, &A) & split_scaled(J12, k, &B) & split_scaled(J21, k, &C) &
            split_scaled(J22, k, &D) & split_scaled(kap, kk, &kp) & split_scaled(Q, kq, &qp) &
            split_scaled(P6, 0, &p6) & split_scaled(1.0 / 6.0, 0, &sixth);
  if (!ok) return false;
  const f2 det = f2_sub(f2_mul(A, D), f2_mul(C, B));
  if (!(fabsf(det.hi) >= 0.25f)) return false;
  const f2 q11 = f2_add_same_sign(f2_mul(D, D), f2_mul(B, B));
  const f2 q22 = f2_add_same_sign(f2_mul(C, C), f2_mul(A, A));
  const f2 q12 = f2_add(f2_mul(D, C), f2_mul(B, A));
  const f2 u = f2_sub(q11, q12), v = f2_sub(q22, q12);
  const f2 s = f2_div(kp, det);
  const f2 s6 = f2_mul(s, sixth);
  bs[0] = join_scaled(f2_mul(f2_add(u, v), s), kk - 1);
  bs[1] = join_scaled(f2_mul(u, s6), kk);
  bs[2] = join_scaled(f2_mul(q11, s), kk - 1);
  bs[3] = join_scaled(f2_mul(v, s6), kk);
  bs[4] = join_scaled(f2_mul(q12, s6), kk);
  bs[5] = join_scaled(f2_mul(q22, s), kk - 1);
  bs[6] = join_scaled(f2_mul(f2_add(u, q22), s6), kk + 3);
  bs[7] = join_scaled(f2_mul(f2_mul(qp, det), p6), kq + 2 * k);
  return true;
}

__device__ __forceinline__ void t6r_bases(double J11, double J12, double J21, double J22, double kap, double Q,
                                          double P6, double* b) {
  if (!t6r_bases_pair(J11, J12, J21, J22, kap, Q, P6, b)) t6r_bases_fp64(J11, J12, J21, J22, kap, Q, P6, b);
}

// The full K (21) and F (6) records from the bases (written out entry by
// entry, so that the bases stay in registers).
template <int LD>
__device__ __forceinline__ void t6r_expand(const double* b, double* a, double* fa) {
  const double m1 = t6r_scale(b[1], 1), m4 = t6r_scale(b[4], 1), m3 = t6r_scale(b[3], 1);
  a[0 * LD] = b[0];
  a[1 * LD] = b[1];
  a[2 * LD] = b[2];
  a[3 * LD] = b[3];
  a[4 * LD] = b[4];
  a[5 * LD] = b[5];
  a[6 * LD] = m1;
  a[7 * LD] = m1;
  a[8 * LD] = 0.0;
  a[9 * LD] = b[6];
  a[10 * LD] = 0.0;
  a[11 * LD] = m4;
  a[12 * LD] = m4;
  a[13 * LD] = t6r_scale(b[3], 2);
  a[14 * LD] = b[6];
  a[15 * LD] = m3;
  a[16 * LD] = 0.0;
  a[17 * LD] = m3;
  a[18 * LD] = t6r_scale(b[4], 2);
  a[19 * LD] = t6r_scale(b[1], 2);
  a[20 * LD] = b[6];
  fa[0 * LD] = 0.0;
  fa[1 * LD] = 0.0;
  fa[2 * LD] = 0.0;
  fa[3 * LD] = b[7];
  fa[4 * LD] = b[7];
  fa[5 * LD] = b[7];
}

// Records of one straight-sided element from its three vertices (reference-
// tensor form): ke = c11 S11 + c22 S22 + c12 (S12 + S21), fe = Q det P.
template <int NN, int LD, int PAT>
__device__ __forceinline__ void straight_record(double x0, double y0, double x1, double y1, double x2, double y2,
                                                double kap, double Q, const double (*sS)[NN * (NN + 1) / 2],
                                                const QPTab& tab, double* acc, double* fa, int t) {
  // Every operation is spelled out (no contraction left to the compiler), so
  // all kernels that inline this produce the same bits.
  constexpr int NS = NN * (NN + 1) / 2;
  const double J11 = __dsub_rn(x1, x0), J12 = __dsub_rn(x2, x0);
  const double J21 = __dsub_rn(y1, y0), J22 = __dsub_rn(y2, y0);
  if (PAT == kPatT6R) {
    double bs[8];
    t6r_bases(J11, J12, J21, J22, kap, Q, tab.P[3], bs);
    t6r_expand<LD>(bs, acc + t, fa + t);
    return;
  }
  const double det = __fma_rn(J11, J22, -__dmul_rn(J21, J12));
  const double s = __ddiv_rn(kap, det);
  const double c11 = __dmul_rn(__fma_rn(J22, J22, __dmul_rn(J12, J12)), s);
  const double c22 = __dmul_rn(__fma_rn(J21, J21, __dmul_rn(J11, J11)), s);
  const double c12 = -__dmul_rn(__fma_rn(J22, J21, __dmul_rn(J12, J11)), s);
  const double qd = __dmul_rn(Q, det);
  if (PAT == kPatT6) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      double a = 0.0;
      if ((kT6S12 >> k) & 1u) a = __dmul_rn(c12, sS[2][k]);
      if ((kT6S22 >> k) & 1u) a = __fma_rn(c22, sS[1][k], a);
      if ((kT6S11 >> k) & 1u) a = __fma_rn(c11, sS[0][k], a);
      acc[k * LD + t] = a;
    }
#pragma unroll
    for (int j = 0; j < NN; ++j) fa[j * LD + t] = ((kT6P >> j) & 1u) ? __dmul_rn(qd, tab.P[j]) : 0.0;
  } else {
#pragma unroll
    for (int k = 0; k < NS; ++k)
      acc[k * LD + t] = __fma_rn(c11, sS[0][k], __fma_rn(c22, sS[1][k], __dmul_rn(c12, sS[2][k])));
#pragma unroll
    for (int j = 0; j < NN; ++j) fa[j * LD + t] = __dmul_rn(qd, tab.P[j]);
  }
}

// The reference tensors' stored entries (column-packed upper triangle) of a CTA.
template <int NN, int NT>
__device__ __forceinline__ void stage_tensors(const QPTab& tab, double (*sS)[NN * (NN + 1) / 2]) {
  constexpr int NS = NN * (NN + 1) / 2;
  for (int k = threadIdx.x; k < NS; k += NT) {
    int j = 0;
    while ((j + 1) * (j + 2) / 2 <= k) ++j;
    int i = k - j * (j + 1) / 2;
    sS[0][k] = tab.S[0][0][i * 6 + j];
    sS[1][k] = tab.S[1][1][i * 6 + j];
    sS[2][k] = tab.S[0][1][i * 6 + j] + tab.S[1][0][i * 6 + j];
  }
}

// The NT elements e0 .. e0 + NT - 1 of one mesh, one per thread.  straight:
// per-element flags (straight_k); PAT: the tensors' zero pattern.
template <int NN, int NT, int PAT>
__device__ __forceinline__ void heat_elems(int64_t e0, int64_t nel, const int32_t* __restrict__ conn,
                                           const double2* __restrict__ xy, const double* __restrict__ kappa, double Q,
                                           const uint8_t* __restrict__ straight, const QPTab& tab,
                                           double* __restrict__ kstore, double* __restrict__ fstore) {
  constexpr int NS = NN * (NN + 1) / 2;
  constexpr int LD = NT + 1;
  extern __shared__ double acc[];  // (NS + NN) * LD
  __shared__ SmemTab st;
  __shared__ int32_t sconn[NT * NN];
  __shared__ double sS[3][NS];
  stage_tables(tab, &st);
  stage_tensors<NN, NT>(tab, sS);
  Geo<NN> g;
  load_geo<NN, NT>(conn, xy, e0, nel, sconn, g, nullptr);  // contains __syncthreads
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  double* fa = acc + NS * LD;
  if (e < nel) {
    const double kap = kappa[e];
    if (NN == 3 || straight[e]) {
      straight_record<NN, LD, PAT>(g.x[0], g.y[0], g.x[1], g.y[1], g.x[2], g.y[2], kap, Q, sS, tab, acc, fa, t);
    } else {
      double ke[NS], fe[NN];
#pragma unroll
      for (int k = 0; k < NS; ++k) ke[k] = 0.0;
#pragma unroll
      for (int j = 0; j < NN; ++j) fe[j] = 0.0;
      for (int q = 0; q < tab.npts; ++q) {
        double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          J11 += g.x[j] * st.G[q][j][0];
          J12 += g.x[j] * st.G[q][j][1];
          J21 += g.y[j] * st.G[q][j][0];
          J22 += g.y[j] * st.G[q][j][1];
        }
        const double det = J11 * J22 - J21 * J12;
        const double rd = 1.0 / det;
        double gx[NN], gy[NN];
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          const double a = st.G[q][j][0], b = st.G[q][j][1];
          gx[j] = (a * J22 - b * J21) * rd;
          gy[j] = (-a * J12 + b * J11) * rd;
        }
        const double JxW = det * st.w[q];
        const double c = kap * JxW;
#pragma unroll
        for (int j = 0; j < NN; ++j) {
#pragma unroll
          for (int i = 0; i <= j; ++i) ke[j * (j + 1) / 2 + i] += (gx[i] * gx[j] + gy[i] * gy[j]) * c;
          fe[j] += st.N[q][j] * Q * JxW;
        }
      }
#pragma unroll
      for (int k = 0; k < NS; ++k) acc[k * LD + t] = ke[k];
#pragma unroll
      for (int j = 0; j < NN; ++j) fa[j * LD + t] = fe[j];
    }
  }
  write_records<NT>(acc, NS, e0, nel, kstore);
  __syncthreads();
  write_records<NT>(fa, NN, e0, nel, fstore);
}

// T6 meshes whose elements are all straight-sided (no curved element in the
// geometry): only the three vertices are gathered and the per-point branch is
// absent, which keeps the register count, and with it the occupancy, of the
// triangle kernel.  Same records, bit for bit, as heat_k's straight branch.
//
// FDIRECT (exact-rule form only): the load vector is added into the global
// vector fglob (zeroed beforehand) instead of being written as records.  The
// exact element load is zero at the vertices and Q det / 6 at the three
// midside nodes, and the caller guarantees that no DOF is a midside node of
// more than two elements.  An IEEE sum of at most two terms onto +0 does not
// depend on their order ((0 + a) + b == (0 + b) + a, signed zeros included),
// so the atomic additions give the bits of the in-order vector assembly.
//
// BASES (exact-rule form only): the 8 bases of each element are written as
// one 64-byte record (kstore: nel x 8) instead of the 21 K values; the tile
// reduction (tiles.cu) expands them to the same values, bit for bit.  With
// the load vector added in place as well, heat_t6_bases_k does this work.
template <int PAT, bool FDIRECT = false, bool BASES = false>
__global__ void __launch_bounds__(kIntThreads) heat_t6s_k(int64_t nel, const int32_t* __restrict__ conn,
                                                         const double2* __restrict__ xy,
                                                         const double* __restrict__ kappa, double Q,
                                                         const __grid_constant__ QPTab tab,
                                                         double* __restrict__ kstore, double* __restrict__ fstore,
                                                         const int32_t* __restrict__ dofs = nullptr,
                                                         double* __restrict__ fglob = nullptr) {
  constexpr int NN = 6, NS = 21, NT = kIntThreads, LD = NT + 1;
  extern __shared__ double acc[];  // (NS + NN) * LD
  __shared__ int32_t sconn[NT * NN];
  __shared__ double sS[3][NS];
  if (PAT != kPatT6R) stage_tensors<NN, NT>(tab, sS);  // the exact-rational form needs no tensors
  const int64_t e0 = (int64_t)blockIdx.x * NT;
  const int64_t base = e0 * NN, lim = nel * NN;
  for (int k = threadIdx.x; k < NT * NN; k += NT) {
    const int64_t gi = base + k;
    sconn[k] = gi < lim ? __ldg(conn + gi) : 0;
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  if (PAT == kPatT6R) {
    // The 8 bases stay in registers; the 27 record values are staged and
    // written in three parts through an 11-entry buffer, which keeps the
    // shared memory per CTA (and with it the occupancy limit) small.
    double bs[8];
    if (e < nel) {
      const double2 p0 = __ldg(xy + sconn[t * NN]), p1 = __ldg(xy + sconn[t * NN + 1]),
                    p2 = __ldg(xy + sconn[t * NN + 2]);
      t6r_bases(__dsub_rn(p1.x, p0.x), __dsub_rn(p2.x, p0.x), __dsub_rn(p1.y, p0.y), __dsub_rn(p2.y, p0.y), kappa[e],
                Q, tab.P[3], bs);
    }
    double* a = acc + t;
    if (BASES) {
      if (e < nel) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k * LD] = bs[k];
      }
      write_records_fixed<NT, 8, 8>(acc, 0, e0, nel, kstore);
      if (FDIRECT) {
        if (e < nel) {
          const int32_t* d = dofs + e * NN;
          atomicAdd(fglob + __ldg(d + 3), bs[7]);
          atomicAdd(fglob + __ldg(d + 4), bs[7]);
          atomicAdd(fglob + __ldg(d + 5), bs[7]);
        }
        return;
      }
      __syncthreads();
      if (e < nel) {
        a[0 * LD] = 0.0;
        a[1 * LD] = 0.0;
        a[2 * LD] = 0.0;
        a[3 * LD] = bs[7];
        a[4 * LD] = bs[7];
        a[5 * LD] = bs[7];
      }
      write_records_part<NT>(acc, NN, 0, NN, e0, nel, fstore);
      return;
    }
    if (e < nel) {
      const double m1 = t6r_scale(bs[1], 1);
      a[0 * LD] = bs[0];
      a[1 * LD] = bs[1];
      a[2 * LD] = bs[2];
      a[3 * LD] = bs[3];
      a[4 * LD] = bs[4];
      a[5 * LD] = bs[5];
      a[6 * LD] = m1;
      a[7 * LD] = m1;
      a[8 * LD] = 0.0;
      a[9 * LD] = bs[6];
      a[10 * LD] = 0.0;
    }
    write_records_fixed<NT, NS, 11>(acc, 0, e0, nel, kstore);
    __syncthreads();
    if (e < nel) {
      const double m4 = t6r_scale(bs[4], 1), m3 = t6r_scale(bs[3], 1);
      a[0 * LD] = m4;                       // 11
      a[1 * LD] = m4;                       // 12
      a[2 * LD] = t6r_scale(bs[3], 2);      // 13
      a[3 * LD] = bs[6];                    // 14
      a[4 * LD] = m3;                       // 15
      a[5 * LD] = 0.0;                      // 16
      a[6 * LD] = m3;                       // 17
      a[7 * LD] = t6r_scale(bs[4], 2);      // 18
      a[8 * LD] = t6r_scale(bs[1], 2);      // 19
      a[9 * LD] = bs[6];                    // 20
    }
    write_records_fixed<NT, NS, 10>(acc, 11, e0, nel, kstore);
    if (FDIRECT) {
      if (e < nel) {
        const int32_t* d = dofs + e * NN;
        atomicAdd(fglob + __ldg(d + 3), bs[7]);
        atomicAdd(fglob + __ldg(d + 4), bs[7]);
        atomicAdd(fglob + __ldg(d + 5), bs[7]);
      }
      return;
    }
    __syncthreads();
    if (e < nel) {
      a[0 * LD] = 0.0;
      a[1 * LD] = 0.0;
      a[2 * LD] = 0.0;
      a[3 * LD] = bs[7];
      a[4 * LD] = bs[7];
      a[5 * LD] = bs[7];
    }
    write_records_part<NT>(acc, NN, 0, NN, e0, nel, fstore);
    return;
  }
  double* fa = acc + NS * LD;
  if (e < nel) {
    const double2 p0 = __ldg(xy + sconn[t * NN]), p1 = __ldg(xy + sconn[t * NN + 1]),
                  p2 = __ldg(xy + sconn[t * NN + 2]);
    straight_record<NN, LD, PAT>(p0.x, p0.y, p1.x, p1.y, p2.x, p2.y, kappa[e], Q, sS, tab, acc, fa, t);
  }
  write_records<NT>(acc, NS, e0, nel, kstore);
  __syncthreads();
  write_records<NT>(fa, NN, e0, nel, fstore);
}

template <int NN, int PAT>
__global__ void __launch_bounds__(kIntThreads) heat_k(int64_t nel, const int32_t* __restrict__ conn,
                                                     const double2* __restrict__ xy, const double* __restrict__ kappa,
                                                     double Q, const uint8_t* __restrict__ straight,
                                                     const __grid_constant__ QPTab tab, double* __restrict__ kstore,
                                                     double* __restrict__ fstore) {
  heat_elems<NN, kIntThreads, PAT>((int64_t)blockIdx.x * kIntThreads, nel, conn, xy, kappa, Q, straight, tab, kstore,
                                   fstore);
}

// Many meshes in one launch: CTA b works on mesh k with jobs[k].blk0 <= b <
// jobs[k + 1].blk0, elements (b - blk0) * NT onwards.
template <int NN, int NT, int PAT>
__global__ void __launch_bounds__(NT) heat_batch_k(const HeatJob* __restrict__ jobs, int njobs,
                                                   const __grid_constant__ QPTab tab) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {  // last job with blk0 <= blockIdx.x
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].blk0 <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
  }
  const HeatJob J = jobs[lo];
  heat_elems<NN, NT, PAT>(((int64_t)blockIdx.x - J.blk0) * NT, J.nel, J.conn, (const double2*)J.xy, J.kappa, J.Q,
                          J.straight, tab, J.kstore, J.fstore);
}

static size_t heat_smem(int nn, int nt) { return (size_t)(nn == 3 ? 6 + 3 : 21 + 6) * (nt + 1) * sizeof(double); }

bool heat_bases_ok(int nn, int64_t ncurved, const QPTab& tab) {
  return nn == 6 && ncurved == 0 && heat_pattern(6, tab) == kPatT6R;
}

// The 8 bases of straight-sided exact-rule T6 elements with the load vector
// added in place (the work of heat_t6s_k<kPatT6R, true, true>), without
// shared memory or barriers: a grid-stride loop in which each thread loads
// the vertex numbers and conductivity of its element two iterations ahead and
// gathers the vertex coordinates one iteration ahead, so that both global
// latencies overlap the float-pair arithmetic of the current element.  The
// bases are those of t6r_bases, bit for bit, and the load-vector additions
// are the same (at most two onto +0 per DOF, order-independent).
__global__ void __launch_bounds__(kIntThreads) heat_t6_bases_k(int64_t nel, const int32_t* __restrict__ conn,
                                                              const double2* __restrict__ xy,
                                                              const double* __restrict__ kappa, double Q, double P6,
                                                              double* __restrict__ bases,
                                                              const int32_t* __restrict__ dofs,
                                                              double* __restrict__ fglob) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nel) return;
  // element e: coordinates and conductivity; element e + stride: vertex numbers and conductivity
  int32_t v0 = __ldg(conn + e * 6), v1 = __ldg(conn + e * 6 + 1), v2 = __ldg(conn + e * 6 + 2);
  double kap = __ldg(kappa + e);
  double2 p0 = __ldg(xy + v0), p1 = __ldg(xy + v1), p2 = __ldg(xy + v2);
  int64_t en = e + stride;
  double kapn = 0.0;
  if (en < nel) {
    v0 = __ldg(conn + en * 6);
    v1 = __ldg(conn + en * 6 + 1);
    v2 = __ldg(conn + en * 6 + 2);
    kapn = __ldg(kappa + en);
  }
  for (;;) {
    // the next element's coordinates, and the vertex numbers of the one after it
    double2 q0 = p0, q1 = p1, q2 = p2;
    const int64_t enn = en + stride;
    double kapnn = 0.0;
    if (en < nel) {
      q0 = __ldg(xy + v0);
      q1 = __ldg(xy + v1);
      q2 = __ldg(xy + v2);
      if (enn < nel) {
        v0 = __ldg(conn + enn * 6);
        v1 = __ldg(conn + enn * 6 + 1);
        v2 = __ldg(conn + enn * 6 + 2);
        kapnn = __ldg(kappa + enn);
      }
    }
    double bs[8];
    t6r_bases(__dsub_rn(p1.x, p0.x), __dsub_rn(p2.x, p0.x), __dsub_rn(p1.y, p0.y), __dsub_rn(p2.y, p0.y), kap, Q, P6,
              bs);
    double2* o = reinterpret_cast<double2*>(bases + e * 8);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = make_double2(bs[2 * k], bs[2 * k + 1]);
    const int32_t* d = dofs + e * 6;
    atomicAdd(fglob + __ldg(d + 3), bs[7]);
    atomicAdd(fglob + __ldg(d + 4), bs[7]);
    atomicAdd(fglob + __ldg(d + 5), bs[7]);
    if (en >= nel) break;
    e = en;
    en = enn;
    p0 = q0;
    p1 = q1;
    p2 = q2;
    kap = kapn;
    kapn = kapnn;
  }
}

int launch_heat_bases(Ctx* c, int64_t nel, const int32_t* conn, const double* xy, const double* kappa, double Q,
                      const QPTab& tab, double* bases, double* fstore, const int32_t* dofs, double* fglob) {
  if (nel == 0) return ELFEL_OK;
  const unsigned grid = grid_for(nel, kIntThreads);
  const size_t sm = 11 * (kIntThreads + 1) * sizeof(double);
  if (fglob) {
    if (!dofs) return fail(c, ELFEL_ERR_STATE, "heat: direct load-vector assembly needs the DOF table");
    // 24 CTAs per SM (6 resident at 77 registers): 0.090 ms at 2M elements;
    // 8, 12, 16, 32, 64: 0.099, 0.095, 0.090, 0.090, 0.094 ms
    const unsigned g = grid_for(nel, kIntThreads, (int64_t)c->sm_count * 24);
    heat_t6_bases_k<<<g, kIntThreads, 0, c->stream>>>(nel, conn, (const double2*)xy, kappa, Q, tab.P[3], bases, dofs,
                                                     fglob);
  } else {
    heat_t6s_k<kPatT6R, false, true><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, kappa, Q,
                                                                            tab, bases, fstore);
  }
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

bool heat_f_direct(int nn, int64_t ncurved, const QPTab& tab) {
  return nn == 6 && ncurved == 0 && heat_pattern(6, tab) == kPatT6R;
}

int launch_heat(Ctx* c, int nn, int64_t nel, const int32_t* conn, const double* xy, const double* kappa, double Q,
                const uint8_t* straight, int64_t ncurved, const QPTab& tab, double* kstore, double* fstore,
                const int32_t* dofs, double* fglob) {
  if (nel == 0) return ELFEL_OK;
  const unsigned grid = grid_for(nel, kIntThreads);
  const double2* p = (const double2*)xy;
  const size_t sm = heat_smem(nn, kIntThreads);
  const int pat = nn == 6 ? heat_pattern(6, tab) : kPatGeneric;
  if (fglob) {
    if (!heat_f_direct(nn, ncurved, tab) || !dofs)
      return fail(c, ELFEL_ERR_STATE, "heat: direct load-vector assembly needs the straight-sided exact T6 form");
    heat_t6s_k<kPatT6R, true><<<grid, kIntThreads, 11 * (kIntThreads + 1) * sizeof(double), c->stream>>>(
        nel, conn, p, kappa, Q, tab, kstore, fstore, dofs, fglob);
    ELFEL_LAUNCH_CHECK(c);
    return ELFEL_OK;
  }
  if (nn == 3)
    heat_k<3, kPatGeneric><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, p, kappa, Q, straight, tab, kstore, fstore);
  else if (ncurved == 0 && pat == kPatT6R)
    heat_t6s_k<kPatT6R><<<grid, kIntThreads, 11 * (kIntThreads + 1) * sizeof(double), c->stream>>>(
        nel, conn, p, kappa, Q, tab, kstore, fstore);
  else if (ncurved == 0 && pat == kPatT6)
    heat_t6s_k<kPatT6><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, p, kappa, Q, tab, kstore, fstore);
  else if (ncurved == 0)
    heat_t6s_k<kPatGeneric><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, p, kappa, Q, tab, kstore, fstore);
  else if (pat == kPatT6R)
    heat_k<6, kPatT6R><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, p, kappa, Q, straight, tab, kstore, fstore);
  else if (pat == kPatT6)
    heat_k<6, kPatT6><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, p, kappa, Q, straight, tab, kstore, fstore);
  else
    heat_k<6, kPatGeneric><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, p, kappa, Q, straight, tab, kstore, fstore);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

// ------------------------------------------------------------------ Q4 / T4 heat
// The reference's integrate! loop (test/test_heat.jl:151-171,
// examples/heat/poisson/t4.jl:32-52) with the quadrature sum kept per point:
//   ke_ij += gradN_i . gradN_j * kappa * det J * w_q,  fe_j += N_j * Q * det J * w_q.
// gradN = gradNpar J^-1 is written as adj(J)-rows / det J, so that
//   ke_ij += (a_i . a_j) * kappa * w_q / det J   (a_i = gradNpar_i adj(J)).
// Q4: J varies over the element; 2-D coordinates.  T4: J is constant, so the
// sum over the points collapses to W = sum_q w_q; 3-D coordinates.
int make_shape_tables(int shape, int npts, const double* pc, const double* w, ShapeTab* t) {
  if (npts < 1 || npts > kMaxQP || (shape != ELFEL_SHAPE_Q4 && shape != ELFEL_SHAPE_T4)) return ELFEL_ERR_ARG;
  memset(t, 0, sizeof(*t));
  t->shape = shape;
  t->npts = npts;
  for (int q = 0; q < npts; ++q) {
    t->w[q] = w[q];
    t->W += w[q];
    if (shape == ELFEL_SHAPE_Q4) {
      const double x = pc[2 * q], y = pc[2 * q + 1];
      const double N[4] = {0.25 * (1.0 - x) * (1.0 - y), 0.25 * (1.0 + x) * (1.0 - y), 0.25 * (1.0 + x) * (1.0 + y),
                           0.25 * (1.0 - x) * (1.0 + y)};
      const double G[4][2] = {{-(1.0 - y) * 0.25, -(1.0 - x) * 0.25},
                              {(1.0 - y) * 0.25, -(1.0 + x) * 0.25},
                              {(1.0 + y) * 0.25, (1.0 + x) * 0.25},
                              {-(1.0 + y) * 0.25, (1.0 - x) * 0.25}};
      for (int j = 0; j < 4; ++j) {
        t->N[q][j] = N[j];
        t->G[q][j][0] = G[j][0];
        t->G[q][j][1] = G[j][1];
      }
    } else {
      const double r = pc[3 * q], s = pc[3 * q + 1], u = pc[3 * q + 2];
      t->N[q][0] = 1.0 - r - s - u;
      t->N[q][1] = r;
      t->N[q][2] = s;
      t->N[q][3] = u;
    }
  }
  for (int j = 0; j < 4; ++j) {
    double P = 0.0;
    for (int q = 0; q < npts; ++q) P += t->w[q] * t->N[q][j];
    t->P[j] = P;
  }
  return ELFEL_OK;
}

constexpr int kShapeNS = 10;  // stored entries of a symmetric 4 x 4 element matrix

template <int NT>
__device__ __forceinline__ void load_conn4(const int32_t* __restrict__ conn, int64_t e0, int64_t nel, int32_t* sconn) {
  const int64_t base = e0 * 4, lim = nel * 4;
  for (int k = threadIdx.x; k < NT * 4; k += NT) {
    const int64_t gi = base + k;
    sconn[k] = gi < lim ? __ldg(conn + gi) : 0;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kIntThreads) heat_q4_k(int64_t nel, const int32_t* __restrict__ conn,
                                                        const double2* __restrict__ xy,
                                                        const double* __restrict__ kappa, double Q,
                                                        const __grid_constant__ ShapeTab tab,
                                                        double* __restrict__ kstore, double* __restrict__ fstore) {
  constexpr int NT = kIntThreads, LD = NT + 1;
  __shared__ double acc[(kShapeNS + 4) * LD];
  __shared__ int32_t sconn[NT * 4];
  const int64_t e0 = (int64_t)blockIdx.x * NT;
  load_conn4<NT>(conn, e0, nel, sconn);
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  double* fa = acc + kShapeNS * LD;
  if (e < nel) {
    double x[4], y[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double2 p = __ldg(xy + sconn[t * 4 + j]);
      x[j] = p.x;
      y[j] = p.y;
    }
    const double kap = kappa[e];
    double ke[kShapeNS], fe[4];
#pragma unroll
    for (int k = 0; k < kShapeNS; ++k) ke[k] = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) fe[j] = 0.0;
    for (int q = 0; q < tab.npts; ++q) {
      double J11 = 0.0, J12 = 0.0, J21 = 0.0, J22 = 0.0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        J11 = fma(x[j], tab.G[q][j][0], J11);
        J12 = fma(x[j], tab.G[q][j][1], J12);
        J21 = fma(y[j], tab.G[q][j][0], J21);
        J22 = fma(y[j], tab.G[q][j][1], J22);
      }
      const double det = J11 * J22 - J21 * J12;
      double u[4], v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double a = tab.G[q][j][0], b = tab.G[q][j][1];
        u[j] = a * J22 - b * J21;
        v[j] = b * J11 - a * J12;
      }
      const double cq = kap * tab.w[q] / det;
      const double fq = Q * det * tab.w[q];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int i = 0; i <= j; ++i) ke[j * (j + 1) / 2 + i] = fma(fma(u[i], u[j], v[i] * v[j]), cq, ke[j * (j + 1) / 2 + i]);
        fe[j] = fma(tab.N[q][j], fq, fe[j]);
      }
    }
#pragma unroll
    for (int k = 0; k < kShapeNS; ++k) acc[k * LD + t] = ke[k];
#pragma unroll
    for (int j = 0; j < 4; ++j) fa[j * LD + t] = fe[j];
  }
  write_records<NT>(acc, kShapeNS, e0, nel, kstore);
  __syncthreads();
  write_records<NT>(fa, 4, e0, nel, fstore);
}

__global__ void __launch_bounds__(kIntThreads) heat_t4_k(int64_t nel, const int32_t* __restrict__ conn,
                                                        const double* __restrict__ xyz,
                                                        const double* __restrict__ kappa, double Q,
                                                        const __grid_constant__ ShapeTab tab,
                                                        double* __restrict__ kstore, double* __restrict__ fstore) {
  constexpr int NT = kIntThreads, LD = NT + 1;
  __shared__ double acc[(kShapeNS + 4) * LD];
  __shared__ int32_t sconn[NT * 4];
  const int64_t e0 = (int64_t)blockIdx.x * NT;
  load_conn4<NT>(conn, e0, nel, sconn);
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  double* fa = acc + kShapeNS * LD;
  if (e < nel) {
    double X[4][3];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double* p = xyz + 3 * (int64_t)sconn[t * 4 + j];
      X[j][0] = __ldg(p);
      X[j][1] = __ldg(p + 1);
      X[j][2] = __ldg(p + 2);
    }
    // columns of J: d_a = x_a - x_0 (gradNpar of FEH1_T4 is [-1 -1 -1; I])
    double d[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int k = 0; k < 3; ++k) d[a][k] = X[a + 1][k] - X[0][k];
    // rows of adj(J): a_1 = d_2 x d_3, a_2 = d_3 x d_1, a_3 = d_1 x d_2; a_0 = -(a_1 + a_2 + a_3)
    double A[4][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double* p = d[(a + 1) % 3];
      const double* r = d[(a + 2) % 3];
      A[a + 1][0] = p[1] * r[2] - p[2] * r[1];
      A[a + 1][1] = p[2] * r[0] - p[0] * r[2];
      A[a + 1][2] = p[0] * r[1] - p[1] * r[0];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) A[0][k] = -(A[1][k] + A[2][k] + A[3][k]);
    const double det = d[0][0] * A[1][0] + d[0][1] * A[1][1] + d[0][2] * A[1][2];
    const double c = kappa[e] * tab.W / det;
    const double qd = Q * det;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int i = 0; i <= j; ++i)
        acc[(j * (j + 1) / 2 + i) * LD + t] = (A[i][0] * A[j][0] + A[i][1] * A[j][1] + A[i][2] * A[j][2]) * c;
      fa[j * LD + t] = qd * tab.P[j];
    }
  }
  write_records<NT>(acc, kShapeNS, e0, nel, kstore);
  __syncthreads();
  write_records<NT>(fa, 4, e0, nel, fstore);
}

int launch_heat_shape(Ctx* c, const ShapeTab& tab, int64_t nel, const int32_t* conn, const double* xy,
                      const double* kappa, double Q, double* kstore, double* fstore) {
  if (nel == 0) return ELFEL_OK;
  const unsigned grid = grid_for(nel, kIntThreads);
  if (tab.shape == ELFEL_SHAPE_Q4)
    heat_q4_k<<<grid, kIntThreads, 0, c->stream>>>(nel, conn, (const double2*)xy, kappa, Q, tab, kstore, fstore);
  else if (tab.shape == ELFEL_SHAPE_T4)
    heat_t4_k<<<grid, kIntThreads, 0, c->stream>>>(nel, conn, xy, kappa, Q, tab, kstore, fstore);
  else
    return fail(c, ELFEL_ERR_ARG, "heat: unknown element shape %d", tab.shape);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

template <int NN, int NT, int PAT>
static void heat_batch_launch(Ctx* c, const HeatJob* jobs, int njobs, int64_t blocks, const QPTab& tab) {
  // T6 with 256-thread CTAs stages more than the default 48 KB of dynamic shared memory
  cudaFuncSetAttribute(heat_batch_k<NN, NT, PAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)heat_smem(NN, NT));
  heat_batch_k<NN, NT, PAT><<<(unsigned)blocks, NT, heat_smem(NN, NT), c->stream>>>(jobs, njobs, tab);
}

template <int NT>
static void heat_batch_launch_nn(Ctx* c, int nn, const HeatJob* jobs, int njobs, int64_t blocks, const QPTab& tab) {
  const int pat = nn == 6 ? heat_pattern(6, tab) : kPatGeneric;
  if (nn == 3) heat_batch_launch<3, NT, kPatGeneric>(c, jobs, njobs, blocks, tab);
  else if (pat == kPatT6R) heat_batch_launch<6, NT, kPatT6R>(c, jobs, njobs, blocks, tab);
  else if (pat == kPatT6) heat_batch_launch<6, NT, kPatT6>(c, jobs, njobs, blocks, tab);
  else heat_batch_launch<6, NT, kPatGeneric>(c, jobs, njobs, blocks, tab);
}

int launch_heat_batch(Ctx* c, int nn, int nt, const HeatJob* jobs_dev, int njobs, int64_t blocks, const QPTab& tab) {
  if (njobs == 0 || blocks == 0) return ELFEL_OK;
  if (blocks > 0x7fffffff) return fail(c, ELFEL_ERR_ARG, "batched heat: too many elements");
  switch (nt) {
    case 64: heat_batch_launch_nn<64>(c, nn, jobs_dev, njobs, blocks, tab); break;
    case 128: heat_batch_launch_nn<128>(c, nn, jobs_dev, njobs, blocks, tab); break;
    case 256: heat_batch_launch_nn<256>(c, nn, jobs_dev, njobs, blocks, tab); break;
    default: return fail(c, ELFEL_ERR_ARG, "batched heat: %d threads per CTA (64, 128 or 256)", nt);
  }
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

// ------------------------------------------------------------------ elasticity
// 2-component vector space; DOF k of the element = node k/2, component k%2.
// B(g,0) = (g1, 0, g2), B(g,1) = (0, g2, g1);  ke_ij += dot(D*B_j, B_i) * JxW.
template <int NN>
__global__ void __launch_bounds__(kIntThreads) elast_k(int64_t nel, const int32_t* __restrict__ conn,
                                                      const double2* __restrict__ xy, const Mat3 D,
                                                      const double* __restrict__ bforce,
                                                      const __grid_constant__ QPTab tab, double* __restrict__ kstore,
                                                      double* __restrict__ fstore) {
  constexpr int ND = 2 * NN;
  constexpr int NS = ND * (ND + 1) / 2;
  constexpr int LD = kIntThreads + 1;
  extern __shared__ double acc[];  // (NS + ND) * LD
  __shared__ SmemTab st;
  __shared__ int32_t sconn[kIntThreads * NN];
  stage_tables(tab, &st);
  const int64_t e0 = (int64_t)blockIdx.x * kIntThreads;
  Geo<NN> g;
  load_geo<NN>(conn, xy, e0, nel, sconn, g, nullptr);
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  double* fa = acc + NS * LD;
  if (e < nel) {
    for (int k = 0; k < NS; ++k) acc[k * LD + t] = 0.0;
    for (int k = 0; k < ND; ++k) fa[k * LD + t] = 0.0;
    double b0 = 0.0, b1 = 0.0;
    if (bforce) {
      b0 = bforce[2 * e];
      b1 = bforce[2 * e + 1];
    }
    for (int q = 0; q < tab.npts; ++q) {
      double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        J11 += g.x[j] * st.G[q][j][0];
        J12 += g.x[j] * st.G[q][j][1];
        J21 += g.y[j] * st.G[q][j][0];
        J22 += g.y[j] * st.G[q][j][1];
      }
      const double det = J11 * J22 - J21 * J12;
      const double rd = 1.0 / det;
      double gx[NN], gy[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        const double a = st.G[q][j][0], b = st.G[q][j][1];
        gx[j] = (a * J22 - b * J21) * rd;
        gy[j] = (-a * J12 + b * J11) * rd;
      }
      const double JxW = det * st.w[q];
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        const int nj = j >> 1;
        double B0, B1, B2;
        if ((j & 1) == 0) { B0 = gx[nj]; B1 = 0.0; B2 = gy[nj]; }
        else { B0 = 0.0; B1 = gy[nj]; B2 = gx[nj]; }
        const double d0 = D.a[0][0] * B0 + D.a[0][1] * B1 + D.a[0][2] * B2;
        const double d1 = D.a[1][0] * B0 + D.a[1][1] * B1 + D.a[1][2] * B2;
        const double d2 = D.a[2][0] * B0 + D.a[2][1] * B1 + D.a[2][2] * B2;
#pragma unroll
        for (int i = 0; i <= j; ++i) {
          const int ni = i >> 1;
          double v;
          if ((i & 1) == 0) v = d0 * gx[ni] + d2 * gy[ni];
          else v = d1 * gy[ni] + d2 * gx[ni];
          acc[(j * (j + 1) / 2 + i) * LD + t] += v * JxW;
        }
      }
      if (bforce) {
#pragma unroll
        for (int a = 0; a < NN; ++a) {
          fa[(2 * a) * LD + t] += st.N[q][a] * b0 * JxW;
          fa[(2 * a + 1) * LD + t] += st.N[q][a] * b1 * JxW;
        }
      }
    }
  }
  write_records(acc, NS, e0, nel, kstore);
  __syncthreads();
  write_records(fa, ND, e0, nel, fstore);
}

// Straight-sided elements (constant Jacobian J, A = J^-1): with the
// parametric gradients G_a(q) the physical ones are G_a(q) A, and
//   ke_(a,c),(b,d) = det J sum_q w_q B_(a,c)^T D B_(b,d)
//                  = sum_(alpha,beta) S^(alpha beta)_ab Phi^cd_(alpha beta),
//   Phi^cd = adj(J) E^cd adj(J)^T / det J,   E^cd = P_c^T D P_d,
// where S are the heat kernel's reference tensors (sum_q w_q G_a,alpha
// G_b,beta) and P_0 g = (g0, 0, g1), P_1 g = (0, g1, g0) build the strain
// vectors: E^00 = [D00 D02; D20 D22], E^01 = [D02 D01; D22 D21],
// E^11 = [D22 D21; D12 D11], E^10 = (E^01)^T.  Four multiply-adds per stored
// entry instead of the per-point loop.  The load vector is det J b P_a.
template <int NN>
__global__ void __launch_bounds__(kIntThreads) elast_straight_k(int64_t nel, const int32_t* __restrict__ conn,
                                                               const double2* __restrict__ xy, const Mat3 D,
                                                               const double* __restrict__ bforce,
                                                               const __grid_constant__ QPTab tab,
                                                               double* __restrict__ kstore,
                                                               double* __restrict__ fstore) {
  constexpr int ND = 2 * NN, NS = ND * (ND + 1) / 2, NP = NN * (NN + 1) / 2;
  constexpr int NT = kIntThreads, LD = NT + 1;
  extern __shared__ double acc[];  // (NS + ND) * LD
  __shared__ int32_t sconn[NT * NN];
  __shared__ double sS[4][NP];  // S^00, S^11, S^01, S^10 of node pairs a <= b, index b(b+1)/2 + a
  for (int k = threadIdx.x; k < NP; k += NT) {
    int b = 0;
    while ((b + 1) * (b + 2) / 2 <= k) ++b;
    const int a = k - b * (b + 1) / 2;
    sS[0][k] = tab.S[0][0][a * 6 + b];
    sS[1][k] = tab.S[1][1][a * 6 + b];
    sS[2][k] = tab.S[0][1][a * 6 + b];
    sS[3][k] = tab.S[1][0][a * 6 + b];
  }
  const int64_t e0 = (int64_t)blockIdx.x * NT;
  const int64_t base = e0 * NN, lim = nel * NN;
  for (int k = threadIdx.x; k < NT * NN; k += NT) {
    const int64_t gi = base + k;
    sconn[k] = gi < lim ? __ldg(conn + gi) : 0;
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  double* fa = acc + NS * LD;
  if (e < nel) {
    const double2 p0 = __ldg(xy + sconn[t * NN]), p1 = __ldg(xy + sconn[t * NN + 1]),
                  p2 = __ldg(xy + sconn[t * NN + 2]);
    const double J11 = p1.x - p0.x, J12 = p2.x - p0.x, J21 = p1.y - p0.y, J22 = p2.y - p0.y;
    const double det = J11 * J22 - J21 * J12;
    const double rd = 1.0 / det;
    // adj(J) = [J22 -J12; -J21 J11];  Phi = adj E adj^T / det
    const double m00 = J22, m01 = -J12, m10 = -J21, m11 = J11;
    double phi[4][4];  // (00, 11, 01, 10) x (alpha beta = 00, 11, 01, 10)
    const double E[3][4] = {{D.a[0][0], D.a[0][2], D.a[2][0], D.a[2][2]},   // E^00 rows
                            {D.a[2][2], D.a[2][1], D.a[1][2], D.a[1][1]},   // E^11
                            {D.a[0][2], D.a[0][1], D.a[2][2], D.a[2][1]}};  // E^01
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const double e00 = E[m][0], e01 = E[m][1], e10 = E[m][2], e11 = E[m][3];
      // T = E adj^T: T_ij = sum_k E_ik adj_jk
      const double t00 = e00 * m00 + e01 * m01, t01 = e00 * m10 + e01 * m11;
      const double t10 = e10 * m00 + e11 * m01, t11 = e10 * m10 + e11 * m11;
      // adj T
      phi[m][0] = (m00 * t00 + m01 * t10) * rd;  // alpha beta = 00
      phi[m][1] = (m10 * t01 + m11 * t11) * rd;  // 11
      phi[m][2] = (m00 * t01 + m01 * t11) * rd;  // 01
      phi[m][3] = (m10 * t00 + m11 * t10) * rd;  // 10
    }
    // Phi^10 = (Phi^01)^T
    phi[3][0] = phi[2][0];
    phi[3][1] = phi[2][1];
    phi[3][2] = phi[2][3];
    phi[3][3] = phi[2][2];
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const int b = j >> 1, dj = j & 1;
#pragma unroll
      for (int i = 0; i <= j; ++i) {
        const int a = i >> 1, ci = i & 1;
        const int cd = ci == dj ? (ci == 0 ? 0 : 1) : (ci == 0 ? 2 : 3);
        // node pair (a, b), a <= b here because i <= j
        const int k = b * (b + 1) / 2 + a;
        acc[(j * (j + 1) / 2 + i) * LD + t] = sS[0][k] * phi[cd][0] + sS[1][k] * phi[cd][1] +
                                             sS[2][k] * phi[cd][2] + sS[3][k] * phi[cd][3];
      }
    }
    double b0 = 0.0, b1 = 0.0;
    if (bforce) {
      b0 = bforce[2 * e];
      b1 = bforce[2 * e + 1];
    }
#pragma unroll
    for (int a = 0; a < NN; ++a) {
      fa[(2 * a) * LD + t] = tab.P[a] * b0 * det;
      fa[(2 * a + 1) * LD + t] = tab.P[a] * b1 * det;
    }
  }
  write_records<NT>(acc, NS, e0, nel, kstore);
  __syncthreads();
  write_records<NT>(fa, ND, e0, nel, fstore);
}

int launch_elasticity(Ctx* c, int nn, int64_t nel, const int32_t* conn, const double* xy, const Mat3& D,
                      const double* bforce, int64_t ncurved, const QPTab& tab, double* kstore, double* fstore) {
  if (nel == 0) return ELFEL_OK;
  const unsigned grid = grid_for(nel, kIntThreads);
  if (ncurved == 0) {
    const size_t sm = (size_t)(nn == 3 ? 21 + 6 : 78 + 12) * (kIntThreads + 1) * sizeof(double);
    if (nn == 3) {
      elast_straight_k<3><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, D, bforce, tab,
                                                                 kstore, fstore);
    } else {
      ELFEL_CUDA(c, cudaFuncSetAttribute(elast_straight_k<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      elast_straight_k<6><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, D, bforce, tab,
                                                                 kstore, fstore);
    }
    ELFEL_LAUNCH_CHECK(c);
    return ELFEL_OK;
  }
  if (nn == 3) {
    const size_t sm = (size_t)(21 + 6) * (kIntThreads + 1) * sizeof(double);
    elast_k<3><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, D, bforce, tab, kstore, fstore);
  } else {
    const size_t sm = (size_t)(78 + 12) * (kIntThreads + 1) * sizeof(double);
    ELFEL_CUDA(c, cudaFuncSetAttribute(elast_k<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    elast_k<6><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, D, bforce, tab, kstore, fstore);
  }
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

// Traction on element edges: consistent nodal loads sum_q w_q N_i(s_q) t |dx/ds|
// with the 3-point Gauss rule on the edge (exact for the quadratic edge).
// Edge k of a triangle runs from vertex k to vertex (k+1)%3; for T6 the
// midside node of that edge is node 3+k.  Output: ntrac records of 2*nen values
// in (edge node, component) order.
__global__ void traction_k(int64_t ntrac, const int32_t* __restrict__ edges /* ntrac x 2: element, local edge */,
                           const int32_t* __restrict__ conn, int nn, const double2* __restrict__ xy, double t0,
                           double t1, double* __restrict__ out) {
  const double gs[3] = {-0.774596669241483377, 0.0, 0.774596669241483377};
  const double gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ntrac; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = edges[2 * k];
    const int le = edges[2 * k + 1];
    const int nen = nn == 6 ? 3 : 2;
    double2 p[3];
    p[0] = xy[conn[e * nn + le]];
    p[1] = xy[conn[e * nn + (le + 1) % 3]];
    if (nen == 3) p[2] = xy[conn[e * nn + 3 + le]];
    double f[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < 3; ++q) {
      const double s = gs[q];
      double N[3], dN[3];
      if (nen == 2) {
        N[0] = 0.5 * (1 - s); N[1] = 0.5 * (1 + s); N[2] = 0;
        dN[0] = -0.5; dN[1] = 0.5; dN[2] = 0;
      } else {
        N[0] = 0.5 * s * (s - 1); N[1] = 0.5 * s * (s + 1); N[2] = 1 - s * s;
        dN[0] = s - 0.5; dN[1] = s + 0.5; dN[2] = -2 * s;
      }
      double tx = 0, ty = 0;
      for (int a = 0; a < nen; ++a) {
        tx += dN[a] * p[a].x;
        ty += dN[a] * p[a].y;
      }
      const double jac = sqrt(tx * tx + ty * ty);
      for (int a = 0; a < nen; ++a) f[a] += gw[q] * N[a] * jac;
    }
    for (int a = 0; a < nen; ++a) {
      out[k * 2 * nen + 2 * a] = f[a] * t0;
      out[k * 2 * nen + 2 * a + 1] = f[a] * t1;
    }
  }
}

int launch_traction(Ctx* c, int64_t ntrac, const int32_t* edges, const int32_t* conn, int nn, const double* xy,
                    double t0, double t1, double* out) {
  if (ntrac == 0) return ELFEL_OK;
  traction_k<<<grid_for(ntrac, 128), 128, 0, c->stream>>>(ntrac, edges, conn, nn, (const double2*)xy, t0, t1, out);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

// ------------------------------------------------------------------ Stokes
// Velocity: vector T6 (12 DOFs, node-major / component-minor), pressure T3.
// Record: kuu upper triangle (78) | kup 12x3 column-major (36).
// kuu_ij += (mu*JxW) * dot(gradNu_i, gradNu_j) when comp(i) == comp(j), else 0
// kup_ij += (-JxW * Np_j) * gradNu_i[comp(i)].
// Also the pressure mass diagonal per element: sum_q w_q det Np_j^2.
__global__ void __launch_bounds__(kIntThreads) stokes_k(int64_t nel, const int32_t* __restrict__ conn,
                                                       const double2* __restrict__ xy, double mu,
                                                       const __grid_constant__ QPTab tab, double* __restrict__ kstore,
                                                       double* __restrict__ pmass) {
  constexpr int NN = 6;
  constexpr int NS = 78;
  constexpr int NR = NS + 36;
  constexpr int LD = kIntThreads + 1;
  extern __shared__ double acc[];  // (NR + 3) * LD
  __shared__ SmemTab st;
  __shared__ int32_t sconn[kIntThreads * NN];
  stage_tables(tab, &st);
  const int64_t e0 = (int64_t)blockIdx.x * kIntThreads;
  Geo<NN> g;
  load_geo<NN>(conn, xy, e0, nel, sconn, g, nullptr);
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  double* pa = acc + NR * LD;
  if (e < nel) {
    double kuu[21];  // scalar Laplacian block (upper triangle), shared by both components
    double kup[12][3];
    double mp[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < 21; ++k) kuu[k] = 0.0;
#pragma unroll
    for (int a = 0; a < 12; ++a) kup[a][0] = kup[a][1] = kup[a][2] = 0.0;
    for (int q = 0; q < tab.npts; ++q) {
      double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        J11 += g.x[j] * st.G[q][j][0];
        J12 += g.x[j] * st.G[q][j][1];
        J21 += g.y[j] * st.G[q][j][0];
        J22 += g.y[j] * st.G[q][j][1];
      }
      const double det = J11 * J22 - J21 * J12;
      const double rd = 1.0 / det;
      double gx[NN], gy[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        const double a = st.G[q][j][0], b = st.G[q][j][1];
        gx[j] = (a * J22 - b * J21) * rd;
        gy[j] = (-a * J12 + b * J11) * rd;
      }
      const double JxW = det * st.w[q];
      const double c = mu * JxW;
#pragma unroll
      for (int j = 0; j < NN; ++j)
#pragma unroll
        for (int i = 0; i <= j; ++i) kuu[j * (j + 1) / 2 + i] += c * (gx[i] * gx[j] + gy[i] * gy[j]);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double s = -JxW * st.Np[q][j];
#pragma unroll
        for (int a = 0; a < NN; ++a) {
          kup[2 * a][j] += s * gx[a];
          kup[2 * a + 1][j] += s * gy[a];
        }
        mp[j] += JxW * st.Np[q][j] * st.Np[q][j];
      }
    }
    // expand the scalar block into the 12x12 upper triangle (cross-component = 0)
#pragma unroll
    for (int J = 0; J < 12; ++J)
#pragma unroll
      for (int I = 0; I <= J; ++I) {
        double v = 0.0;
        if ((I & 1) == (J & 1)) {
          const int i = I >> 1, j = J >> 1;
          v = kuu[j * (j + 1) / 2 + i];
        }
        acc[(J * (J + 1) / 2 + I) * LD + t] = v;
      }
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int a = 0; a < 12; ++a) acc[(NS + a + 12 * j) * LD + t] = kup[a][j];
#pragma unroll
    for (int j = 0; j < 3; ++j) pa[j * LD + t] = mp[j];
  }
  write_records(acc, NR, e0, nel, kstore);
  __syncthreads();
  write_records(pa, 3, e0, nel, pmass);
}

// Straight-sided elements: the scalar Laplacian block is the heat record with
// kappa = mu (straight_record), the velocity-pressure block
//   kup_(a,c),j = -sum_q w_q det Np_j g_a,c = -sum_alpha T^alpha_aj adj(J)_alpha,c
// (T the tabulated sum_q w_q Np_j G_a,alpha, det J g = G adj(J)), and the
// pressure mass det J Mp_j.
template <int PAT>
__global__ void __launch_bounds__(kIntThreads) stokes_straight_k(int64_t nel, const int32_t* __restrict__ conn,
                                                                const double2* __restrict__ xy, double mu,
                                                                const __grid_constant__ QPTab tab,
                                                                double* __restrict__ kstore,
                                                                double* __restrict__ pmass) {
  constexpr int NN = 6, NS = 78, NR = NS + 36, NT = kIntThreads, LD = NT + 1;
  extern __shared__ double acc[];  // (NR + 3 + 21 + 6) * LD
  __shared__ int32_t sconn[NT * NN];
  __shared__ double sS[3][21];
  stage_tensors<NN, NT>(tab, sS);
  const int64_t e0 = (int64_t)blockIdx.x * NT;
  const int64_t base = e0 * NN, lim = nel * NN;
  for (int k = threadIdx.x; k < NT * NN; k += NT) {
    const int64_t gi = base + k;
    sconn[k] = gi < lim ? __ldg(conn + gi) : 0;
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int64_t e = e0 + t;
  double* pa = acc + NR * LD;
  double* kb = pa + 3 * LD;  // the scalar block (21 entries) and an unused load vector (6)
  double* fb = kb + 21 * LD;
  if (e < nel) {
    const double2 p0 = __ldg(xy + sconn[t * NN]), p1 = __ldg(xy + sconn[t * NN + 1]),
                  p2 = __ldg(xy + sconn[t * NN + 2]);
    straight_record<NN, LD, PAT>(p0.x, p0.y, p1.x, p1.y, p2.x, p2.y, mu, 0.0, sS, tab, kb, fb, t);
#pragma unroll
    for (int J = 0; J < 12; ++J)
#pragma unroll
      for (int I = 0; I <= J; ++I) {
        double v = 0.0;
        if ((I & 1) == (J & 1)) v = kb[((J >> 1) * ((J >> 1) + 1) / 2 + (I >> 1)) * LD + t];
        acc[(J * (J + 1) / 2 + I) * LD + t] = v;
      }
    const double J11 = p1.x - p0.x, J12 = p2.x - p0.x, J21 = p1.y - p0.y, J22 = p2.y - p0.y;
    const double det = J11 * J22 - J21 * J12;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
#pragma unroll
      for (int a = 0; a < NN; ++a) {
        const double t0 = tab.T[0][a * 3 + j], t1 = tab.T[1][a * 3 + j];
        acc[(NS + 2 * a + 12 * j) * LD + t] = -(t0 * J22 - t1 * J21);
        acc[(NS + 2 * a + 1 + 12 * j) * LD + t] = -(t1 * J11 - t0 * J12);
      }
      pa[j * LD + t] = det * tab.Mp[j];
    }
  }
  write_records<NT>(acc, NR, e0, nel, kstore);
  __syncthreads();
  write_records<NT>(pa, 3, e0, nel, pmass);
}

int launch_stokes(Ctx* c, int64_t nel, const int32_t* conn, const double* xy, double mu, int64_t ncurved,
                  const QPTab& tab, double* kstore, double* pmass) {
  if (nel == 0) return ELFEL_OK;
  if (ncurved == 0) {
    const size_t sm = (size_t)(78 + 36 + 3 + 21 + 6) * (kIntThreads + 1) * sizeof(double);
    const int pat = heat_pattern(6, tab);
    const unsigned grid = grid_for(nel, kIntThreads);
    if (pat == kPatT6R) {
      ELFEL_CUDA(c, cudaFuncSetAttribute(stokes_straight_k<kPatT6R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sm));
      stokes_straight_k<kPatT6R><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, mu, tab,
                                                                         kstore, pmass);
    } else if (pat == kPatT6) {
      ELFEL_CUDA(c, cudaFuncSetAttribute(stokes_straight_k<kPatT6>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sm));
      stokes_straight_k<kPatT6><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, mu, tab,
                                                                        kstore, pmass);
    } else {
      ELFEL_CUDA(c, cudaFuncSetAttribute(stokes_straight_k<kPatGeneric>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      stokes_straight_k<kPatGeneric><<<grid, kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, mu, tab,
                                                                             kstore, pmass);
    }
    ELFEL_LAUNCH_CHECK(c);
    return ELFEL_OK;
  }
  const size_t sm = (size_t)(78 + 36 + 3) * (kIntThreads + 1) * sizeof(double);
  ELFEL_CUDA(c, cudaFuncSetAttribute(stokes_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  stokes_k<<<grid_for(nel, kIntThreads), kIntThreads, sm, c->stream>>>(nel, conn, (const double2*)xy, mu, tab,
                                                                        kstore, pmass);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

}  // namespace elfel
