// L2 error integrals of a computed field against a polynomial exact solution,
// on the device: evaluate_pressure_error / evaluate_velocity_error of the
// reference (Elfel.jl test/test_stokes.jl:438-496, 716-746), which loop over
// the elements and quadrature points of the field's space, locate each point
// (location, src/FEIterators.jl:227-235), interpolate the field from the
// element's DOF values (eldofvals, :201-214) and add
//   w_q det J (u_h(x_q) - u_exact(x_q))^2,
// summed over the components of a vector field; the result is the square root.
//
// The field's space is the primary space of a fused system (space 0: the
// temperature or velocity, nodes_per_elem 3 or 6) or the Taylor-Hood pressure
// (space 1: T3 on the vertices of the velocity elements, so its geometry is
// the vertex triangle).  Exact solutions are bivariate polynomials of degree
// <= 4 per component, which cover the reference's test solutions.
// One thread per element; block partials and a last-block sum in a fixed
// order, so the result is deterministic.
#include "integrate.cuh"
#include "sysmat.cuh"

namespace elfel {

namespace {

constexpr int kErrThreads = 256;

struct Poly {
  double c[2][15];  // per component: (a,b) = (0,0),(1,0),(0,1),(2,0),(1,1),(0,2),(3,0),...,(0,4)
};

__device__ __forceinline__ double poly_at(const double* c, double x, double y) {
  const double x2 = x * x, y2 = y * y;
  const double x3 = x2 * x, y3 = y2 * y;
  double v = c[0];
  v += c[1] * x + c[2] * y;
  v += c[3] * x2 + c[4] * x * y + c[5] * y2;
  v += c[6] * x3 + c[7] * x2 * y + c[8] * x * y2 + c[9] * y3;
  v += c[10] * x2 * x2 + c[11] * x3 * y + c[12] * x2 * y2 + c[13] * x * y3 + c[14] * y2 * y2;
  return v;
}

// NG: geometry nodes (the space's nodes for space 0; 3 vertices for the
// pressure); NV: value nodes of the space; NC: components.
template <int NG, int NV, int NC>
__global__ void __launch_bounds__(kErrThreads) error_k(int64_t nel, const int32_t* __restrict__ conn, int nn_conn,
                                                      const double2* __restrict__ xy,
                                                      const int32_t* __restrict__ dofs,
                                                      const double* __restrict__ U, const __grid_constant__ QPTab tg,
                                                      const __grid_constant__ QPTab tv, const __grid_constant__ Poly P,
                                                      RedSlot red, double* total) {
  __shared__ double sh[kErrThreads / 32];
  double part = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nel; e += (int64_t)gridDim.x * blockDim.x) {
    double x[NG], y[NG];
#pragma unroll
    for (int j = 0; j < NG; ++j) {
      const double2 p = xy[conn[e * nn_conn + j]];
      x[j] = p.x;
      y[j] = p.y;
    }
    double u[NV][NC];
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
      for (int c = 0; c < NC; ++c) u[j][c] = U[dofs[(e * NV + j) * NC + c]];
    for (int q = 0; q < tg.npts; ++q) {
      double J11 = 0, J12 = 0, J21 = 0, J22 = 0, xq = 0, yq = 0;
#pragma unroll
      for (int j = 0; j < NG; ++j) {
        J11 += x[j] * tg.G[q][j][0];
        J12 += x[j] * tg.G[q][j][1];
        J21 += y[j] * tg.G[q][j][0];
        J22 += y[j] * tg.G[q][j][1];
        xq += x[j] * tg.N[q][j];
        yq += y[j] * tg.N[q][j];
      }
      const double det = J11 * J22 - J21 * J12;
      double d2 = 0.0;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        double uh = 0.0;
#pragma unroll
        for (int j = 0; j < NV; ++j) uh += u[j][c] * tv.N[q][j];
        const double d = uh - poly_at(P.c[c], xq, yq);
        d2 += d * d;
      }
      part += det * tg.w[q] * d2;
    }
  }
  const double s = block_sum<kErrThreads>(part, sh);
  finish_sum(s, red, total);
}

template <int NG, int NV, int NC>
int launch_error(Ctx* c, int64_t nel, const int32_t* conn, int nn_conn, const double* xy, const int32_t* dofs,
                 const double* U, const QPTab& tg, const QPTab& tv, const Poly& P, double* total) {
  RedSlot rs;
  const unsigned grid = grid_for(nel, kErrThreads, (int64_t)kRedBlocks);
  ELFEL_TRY(red_scratch(c, 1, (int)grid, &rs));
  error_k<NG, NV, NC><<<grid, kErrThreads, 0, c->stream>>>(nel, conn, nn_conn, (const double2*)xy, dofs, U, tg, tv,
                                                           P, rs, total);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

}  // namespace

}  // namespace elfel

using namespace elfel;

extern "C" int elfel_error_l2(elfel_sysmat* m, const double* U, int32_t space, const double* poly, int32_t npts,
                              const double* qp_coords, const double* qp_weights, double* err) {
  if (!m || !m->h) return ELFEL_ERR_ARG;
  Ctx* c = &m->h->c;
  if (!m->fused) return fail(c, ELFEL_ERR_STATE, "error_l2: a fused system is required");
  if (!U || !poly || !err || !qp_coords || !qp_weights) return fail(c, ELFEL_ERR_ARG, "error_l2: NULL argument");
  if (npts < 1 || npts > kMaxQP) return fail(c, ELFEL_ERR_ARG, "error_l2: quadrature with %d points", npts);
  const Fused& F = m->F;
  if (F.shape != ELFEL_SHAPE_TRIANGLE)
    return fail(c, ELFEL_ERR_UNSUPPORTED, "error_l2: triangle (T3/T6) spaces only");
  if (space != 0 && !(space == 1 && F.physics == ELFEL_STOKES))
    return fail(c, ELFEL_ERR_ARG, "error_l2: space 0, or 1 (pressure) of a Stokes system");
  cudaSetDevice(c->device);
  Poly P;
  memset(&P, 0, sizeof(P));
  const int ncomp = space == 0 ? F.ncomp_u : 1;
  for (int k = 0; k < ncomp; ++k)
    for (int i = 0; i < 15; ++i) P.c[k][i] = poly[k * 15 + i];
  QPTab tg, tv;
  const int ng = space == 0 ? F.nn_u : 3;
  ELFEL_TRY(make_tables(ng, npts, qp_coords, qp_weights, &tg));
  ELFEL_TRY(make_tables(space == 0 ? F.nn_u : 3, npts, qp_coords, qp_weights, &tv));
  const int64_t n = m->nrow;
  DBuf<double> Ud, tot;
  ELFEL_TRY(Ud.alloc(c, (size_t)(n > 0 ? n : 1)));
  ELFEL_TRY(tot.alloc(c, 1));
  if (n) ELFEL_CUDA(c, cudaMemcpyAsync(Ud.p, U, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  int rc = ELFEL_OK;
  if (space == 1)
    rc = launch_error<3, 3, 1>(c, F.nel, F.conn_u.p, F.nn_u, F.xy_u.p, F.dofs_p.p, Ud.p, tg, tv, P, tot.p);
  else if (F.nn_u == 3 && ncomp == 1)
    rc = launch_error<3, 3, 1>(c, F.nel, F.conn_u.p, 3, F.xy_u.p, F.dofs_u.p, Ud.p, tg, tv, P, tot.p);
  else if (F.nn_u == 3 && ncomp == 2)
    rc = launch_error<3, 3, 2>(c, F.nel, F.conn_u.p, 3, F.xy_u.p, F.dofs_u.p, Ud.p, tg, tv, P, tot.p);
  else if (F.nn_u == 6 && ncomp == 1)
    rc = launch_error<6, 6, 1>(c, F.nel, F.conn_u.p, 6, F.xy_u.p, F.dofs_u.p, Ud.p, tg, tv, P, tot.p);
  else if (F.nn_u == 6 && ncomp == 2)
    rc = launch_error<6, 6, 2>(c, F.nel, F.conn_u.p, 6, F.xy_u.p, F.dofs_u.p, Ud.p, tg, tv, P, tot.p);
  else
    rc = fail(c, ELFEL_ERR_UNSUPPORTED, "error_l2: nodes %d, components %d", F.nn_u, ncomp);
  if (rc != ELFEL_OK) return rc;
  double e2 = 0.0;
  ELFEL_CUDA(c, cudaMemcpyAsync(&e2, tot.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  Ud.release(c);
  tot.release(c);
  *err = sqrt(e2);
  return ELFEL_OK;
}
