// Block meshes generated on the device: the T3block / T6block meshes of
// MeshSteward 1.1.3 that the reference's tests use (e.g. Elfel.jl
// test/test_heat.jl:28-33), and the DOF numbering of a scalar field fixed on
// the whole boundary (setebc! on the boundary nodes, then numberdofs!,
// src/FESpaces.jl:250-259, 287-291: free DOFs first, data DOFs after, each
// in node order).  Every table is closed-form in the grid indices, so no
// host arrays and no scan are needed.
//
// Conventions (the same as the host generators of the Python layer): nodes
// are numbered x-fastest (T6 on the refined (2nx+1) x (2ny+1) grid); cell
// (i, j) is visited with i outer and j inner and split into 2 triangles
// [n1 n2 n3], [n1 n3 n4] of its corners (i,j), (i+1,j), (i+1,j+1), (i,j+1),
// or, in alternate orientation for odd i + j, [n1 n2 n4], [n2 n3 n4]; T6
// midside node k+3 sits on the edge from vertex k to vertex k+1.
// Coordinates are numpy.linspace's: x_i = i * (lx / nx), x_nx = lx, and T6
// midside coordinates 0.5 * (x_i + x_{i+1}).
#include <algorithm>

#include "sysmat.cuh"

namespace elfel {

namespace {

struct Grid {
  int nn, orient, nx, ny, W, H;
  double lx, ly;
};

__device__ __forceinline__ double lin(int i, int n, double L) { return i == n ? L : (double)i * (L / (double)n); }

// coordinate of grid line a (refined grid for T6)
__device__ __forceinline__ double coord(int a, int n, double L, bool t6) {
  if (!t6) return lin(a, n, L);
  if ((a & 1) == 0) return lin(a >> 1, n, L);
  return 0.5 * (lin(a >> 1, n, L) + lin((a >> 1) + 1, n, L));
}

// 0-based DOF of node (a, b): interior nodes are the free DOFs, boundary
// nodes the data DOFs after them, both in node order.
__device__ __forceinline__ int32_t node_dof(const Grid& g, int a, int b) {
  const int64_t nu = (int64_t)(g.W - 2) * (g.H - 2);
  const bool bnd = a == 0 || a == g.W - 1 || b == 0 || b == g.H - 1;
  if (!bnd) return (int32_t)((int64_t)(b - 1) * (g.W - 2) + (a - 1));
  int64_t before;  // interior nodes numbered before (a, b)
  if (b == 0) before = 0;
  else if (b == g.H - 1) before = nu;
  else before = (int64_t)(b - 1) * (g.W - 2) + (a == 0 ? 0 : g.W - 2);
  return (int32_t)(nu + (int64_t)b * g.W + a - before);
}

__global__ void block_nodes_k(Grid g, double2* __restrict__ xy) {
  const int64_t n = (int64_t)g.W * g.H;
  const bool t6 = g.nn == 6;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < n; id += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(id / g.W), a = (int)(id - (int64_t)b * g.W);
    xy[id] = make_double2(coord(a, g.nx, g.lx, t6), coord(b, g.ny, g.ly, t6));
  }
}

__global__ void block_elems_k(Grid g, int32_t* __restrict__ conn, int32_t* __restrict__ dofs) {
  const int64_t ncell = (int64_t)g.nx * g.ny;
  for (int64_t cidx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; cidx < ncell;
       cidx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(cidx / g.ny), j = (int)(cidx - (int64_t)i * g.ny);
    const bool flip = g.orient == 1 && ((i + j) & 1) == 1;
    // corners on the node grid (refined for T6)
    const int s = g.nn == 6 ? 2 : 1;
    const int cx[4] = {s * i, s * i + s, s * i + s, s * i};
    const int cy[4] = {s * j, s * j, s * j + s, s * j + s};
    // vertex corners of the two triangles
    const int t1[3] = {0, 1, flip ? 3 : 2};
    const int t2[3] = {flip ? 1 : 0, 2, 3};
    for (int t = 0; t < 2; ++t) {
      const int* v = t == 0 ? t1 : t2;
      const int64_t e = 2 * cidx + t;
      int px[6], py[6];
      for (int k = 0; k < 3; ++k) {
        px[k] = cx[v[k]];
        py[k] = cy[v[k]];
      }
      if (g.nn == 6)
        for (int k = 0; k < 3; ++k) {
          px[3 + k] = (px[k] + px[(k + 1) % 3]) / 2;
          py[3 + k] = (py[k] + py[(k + 1) % 3]) / 2;
        }
      for (int k = 0; k < g.nn; ++k) {
        conn[e * g.nn + k] = (int32_t)((int64_t)py[k] * g.W + px[k]);
        dofs[e * g.nn + k] = node_dof(g, px[k], py[k]);
      }
    }
  }
}

// T[dof(node)] at the data DOFs; 0 at free DOFs.  Explicitly rounded
// operations, in this order, so no contraction changes the values.
__global__ void block_dirichlet_k(Grid g, const double2* __restrict__ xy, double c0, double c1, double c2, double c3,
                                  double c4, double c5, double* __restrict__ T) {
  const int64_t n = (int64_t)g.W * g.H;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < n; id += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(id / g.W), a = (int)(id - (int64_t)b * g.W);
    const int32_t d = node_dof(g, a, b);
    const bool bnd = a == 0 || a == g.W - 1 || b == 0 || b == g.H - 1;
    double t = 0.0;
    if (bnd) {
      const double x = xy[id].x, y = xy[id].y;
      t = c0;
      t = __dadd_rn(t, __dmul_rn(c1, x));
      t = __dadd_rn(t, __dmul_rn(c2, y));
      t = __dadd_rn(t, __dmul_rn(c3, __dmul_rn(x, x)));
      t = __dadd_rn(t, __dmul_rn(c4, __dmul_rn(x, y)));
      t = __dadd_rn(t, __dmul_rn(c5, __dmul_rn(y, y)));
    }
    T[d] = t;
  }
}

Grid grid_of(const elfel_block_desc& d) {
  Grid g;
  g.nn = d.nodes_per_elem;
  g.orient = d.orientation;
  g.nx = d.nx;
  g.ny = d.ny;
  g.W = d.nodes_per_elem == 6 ? 2 * d.nx + 1 : d.nx + 1;
  g.H = d.nodes_per_elem == 6 ? 2 * d.ny + 1 : d.ny + 1;
  g.lx = d.lx;
  g.ly = d.ly;
  return g;
}

}  // namespace

int block_tables(Ctx* c, const elfel_block_desc& d, Fused* F, int64_t* nu) {
  if ((d.nodes_per_elem != 3 && d.nodes_per_elem != 6) || (d.orientation != 0 && d.orientation != 1))
    return fail(c, ELFEL_ERR_ARG, "block mesh: nodes_per_elem 3 or 6, orientation 0 or 1");
  if (d.nx < 1 || d.ny < 1 || !(d.lx > 0.0) || !(d.ly > 0.0))
    return fail(c, ELFEL_ERR_ARG, "block mesh: nx, ny >= 1 and a rectangle of positive size");
  const Grid g = grid_of(d);
  const int64_t nnodes = (int64_t)g.W * g.H;
  const int64_t nel = 2LL * d.nx * d.ny;
  if (nnodes >= (int64_t)0x7fffffff || nel * d.nodes_per_elem >= (int64_t)0x7fffffff)
    return fail(c, ELFEL_ERR_ARG, "block mesh: too large for 32-bit device indices");
  F->nn_u = d.nodes_per_elem;
  F->ncomp_u = 1;
  F->nel = nel;
  F->nnodes_u = nnodes;
  ELFEL_TRY(F->xy_u.alloc(c, (size_t)(2 * nnodes)));
  ELFEL_TRY(F->conn_u.alloc(c, (size_t)(nel * d.nodes_per_elem)));
  ELFEL_TRY(F->dofs_u.alloc(c, (size_t)(nel * d.nodes_per_elem)));
  block_nodes_k<<<grid_for(nnodes, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(g, (double2*)F->xy_u.p);
  block_elems_k<<<grid_for((int64_t)d.nx * d.ny, 128, (int64_t)c->sm_count * 16), 128, 0, c->stream>>>(
      g, F->conn_u.p, F->dofs_u.p);
  ELFEL_LAUNCH_CHECK(c);
  *nu = (int64_t)(g.W - 2) * (g.H - 2);
  return ELFEL_OK;
}

int block_dirichlet(Ctx* c, const elfel_block_desc& d, const double* k, const Fused& F, double* T) {
  const Grid g = grid_of(d);
  const int64_t n = (int64_t)g.W * g.H;
  block_dirichlet_k<<<grid_for(n, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
      g, (const double2*)F.xy_u.p, k[0], k[1], k[2], k[3], k[4], k[5], T);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

__global__ void to_one_based_k(const int32_t* __restrict__ a, int64_t n, int64_t* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (int64_t)a[i] + 1;
}

int tables_to_host(Ctx* c, const Fused& F, int64_t* conn, double* xy, int64_t* eldofs) {
  const int64_t nc = F.nel * F.nn_u, nd = F.nel * F.nn_u * F.ncomp_u;
  DBuf<int64_t> tmp;
  ELFEL_TRY(tmp.alloc(c, (size_t)std::max<int64_t>(std::max(nc, nd), 1)));
  if (conn && nc) {
    to_one_based_k<<<grid_for(nc, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(F.conn_u.p, nc, tmp.p);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_CUDA(c, cudaMemcpyAsync(conn, tmp.p, sizeof(int64_t) * nc, cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (eldofs && nd) {
    to_one_based_k<<<grid_for(nd, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(F.dofs_u.p, nd, tmp.p);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_CUDA(c, cudaMemcpyAsync(eldofs, tmp.p, sizeof(int64_t) * nd, cudaMemcpyDeviceToHost, c->stream));
  }
  if (xy && F.nnodes_u)
    ELFEL_CUDA(c, cudaMemcpyAsync(xy, F.xy_u.p, sizeof(double) * F.sdim * F.nnodes_u, cudaMemcpyDeviceToHost,
                                  c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  tmp.release(c);
  return ELFEL_OK;
}

}  // namespace elfel
