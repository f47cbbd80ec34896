// C ABI: SysmatAssemblerSparse (COO mode), SysvecAssembler, fused assembly.
#include <math.h>

#include "integrate.cuh"
#include "solve.cuh"
#include "sysmat.cuh"
#include "t6r.cuh"

using namespace elfel;

namespace elfel {

// Dense vector from a 1 x n pattern: out[c] = 0 + the contributions of
// column c in slot order, as SysvecAssembler adds element vectors into a
// zeroed vector (Assemblers.jl:194-207; the leading +0 turns a sum of
// negative zeros into +0, as there).
__global__ void reduce_row0_dense_k(const int64_t* __restrict__ colptr, const int32_t* __restrict__ cptr,
                                    const int32_t* __restrict__ contrib, const double* __restrict__ store, int64_t n,
                                    double* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k0 = colptr[c], k1 = colptr[c + 1];
    double s = 0.0;
    if (k1 > k0) {
      const int32_t b = cptr[k0], e = cptr[k0 + 1];
      s = __dadd_rn(0.0, store[contrib[b]]);
      for (int32_t t = b + 1; t < e; ++t) s += store[contrib[t]];
    }
    out[c] = s;
  }
}

// *many = 1 when some DOF is a midside node (local nodes 3..5) of more than
// two T6 elements; cnt (ndofs, zeroed) counts the occurrences.
__global__ void midside_count_k(const int32_t* __restrict__ dofs, int64_t nel, int32_t* __restrict__ cnt,
                                int32_t* __restrict__ many) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nel * 3; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / 3;
    if (atomicAdd(cnt + dofs[e * 6 + 3 + (i - e * 3)], 1) >= 2) *many = 1;
  }
}

int reduce_dense(Ctx* c, const Pattern& P, const double* store, double* out) {
  if (P.ncol == 0) return ELFEL_OK;
  reduce_row0_dense_k<<<grid_for(P.ncol, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
      P.colptr.p, P.cptr.p, P.contrib.p, store, P.ncol, out);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

__global__ void csc_out_k(const int64_t* colptr, int64_t ncol, const int32_t* rowval, int64_t nnz, int64_t* colptr1,
                          int64_t* rowval1) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= ncol || i < nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i <= ncol) colptr1[i] = colptr[i] + 1;
    if (i < nnz) rowval1[i] = (int64_t)rowval[i] + 1;
  }
}

__global__ void add_k(double* a, const double* b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] += b[i];
}

// Edge DOF table of the traction edges: (edge node a, component) in order.
__global__ void edge_dofs_k(int64_t ntrac, const int32_t* edges, const int32_t* dofs, int nn, int ncomp,
                            int32_t* out) {
  const int nen = nn == 6 ? 3 : 2;
  const int nedof = nn * ncomp;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ntrac; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = edges[2 * k];
    const int le = edges[2 * k + 1];
    for (int a = 0; a < nen; ++a) {
      const int ln = a == 0 ? le : (a == 1 ? (le + 1) % 3 : 3 + le);
      for (int cc = 0; cc < ncomp; ++cc) out[k * nen * ncomp + a * ncomp + cc] = dofs[e * nedof + ln * ncomp + cc];
    }
  }
}

static int ensure_cap(Ctx* c, DBuf<int64_t>* b, size_t used, size_t need) {
  if (need <= b->n) return ELFEL_OK;
  size_t cap = b->n ? b->n : 1024;
  while (cap < need) cap *= 2;
  DBuf<int64_t> nb;
  ELFEL_TRY(nb.alloc(c, cap));
  if (used) ELFEL_CUDA(c, cudaMemcpyAsync(nb.p, b->p, used * sizeof(int64_t), cudaMemcpyDeviceToDevice, c->stream));
  b->release(c);
  *b = nb;
  return ELFEL_OK;
}
static int ensure_cap(Ctx* c, DBuf<double>* b, size_t used, size_t need) {
  if (need <= b->n) return ELFEL_OK;
  size_t cap = b->n ? b->n : 1024;
  while (cap < need) cap *= 2;
  DBuf<double> nb;
  ELFEL_TRY(nb.alloc(c, cap));
  if (used) ELFEL_CUDA(c, cudaMemcpyAsync(nb.p, b->p, used * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  b->release(c);
  *b = nb;
  return ELFEL_OK;
}

__global__ void coo_index_k(const int64_t* src, int64_t n, int64_t limit, int32_t* dst, int* bad) {
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

}  // namespace elfel

// COO staging buffers live with the sysmat (device).
struct CooStage {
  DBuf<int64_t> I, J;
  DBuf<double> V;
  int64_t n = 0;
};

static CooStage* stage_of(elfel_sysmat* m) {
  static_assert(sizeof(CooStage) > 0, "");
  return reinterpret_cast<CooStage*>(m->coo_stage);
}

#define CHECK_M(m)                          \
  do {                                      \
    if (!(m) || !(m)->h) return ELFEL_ERR_ARG; \
  } while (0)

// Calls that change a system refuse while a batch slot holds it.
#define CHECK_FREE(m)                                                                             \
  do {                                                                                            \
    CHECK_M(m);                                                                                   \
    if ((m)->busy) return fail(&(m)->h->c, ELFEL_ERR_STATE, "the system is held by a batch slot"); \
  } while (0)

extern "C" int elfel_sysmat_create(elfel_ctx* h, elfel_sysmat** out) {
  if (!h || !out) return ELFEL_ERR_ARG;
  elfel_sysmat* m = new elfel_sysmat();
  m->h = h;
  m->coo_stage = new CooStage();
  *out = m;
  return ELFEL_OK;
}

static void release_all(elfel_sysmat* m) {
  Ctx* c = &m->h->c;
  CooStage* s = stage_of(m);
  s->I.release(c);
  s->J.release(c);
  s->V.release(c);
  s->n = 0;
  m->P.release(c);
  m->vals.release(c);
  m->rhs.release(c);
  m->F.release(c);
  solver_release(c, m);
  m->has_rhs = 0;
  m->fused = 0;
  m->finished = 0;
  m->pattern_recorded = 0;
}

// Marks m->P complete at this point of the context stream.
static int record_pattern(elfel_sysmat* m) {
  Ctx* c = &m->h->c;
  if (!m->ev_pattern) ELFEL_CUDA(c, cudaEventCreateWithFlags(&m->ev_pattern, cudaEventDisableTiming));
  ELFEL_CUDA(c, cudaEventRecord(m->ev_pattern, c->stream));
  m->pattern_recorded = 1;
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_destroy(elfel_sysmat* m) {
  if (!m) return ELFEL_OK;
  if (m->busy) return fail(&m->h->c, ELFEL_ERR_STATE, "destroy: the system is held by a batch slot");
  if (m->h) {
    cudaSetDevice(m->h->c.device);
    release_all(m);
    cudaStreamSynchronize(m->h->c.stream);
    if (m->ev_pattern) cudaEventDestroy(m->ev_pattern);
  }
  delete stage_of(m);
  delete m;
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_start(elfel_sysmat* m, int64_t nrow, int64_t ncol) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (nrow < 0 || ncol < 0) return fail(c, ELFEL_ERR_ARG, "start!: negative dimensions");
  cudaSetDevice(c->device);
  release_all(m);
  m->nrow = nrow;
  m->ncol = ncol;
  m->started = 1;
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_assemble_coo(elfel_sysmat* m, const int64_t* rows, const int64_t* cols,
                                         const double* vals, int64_t n) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (!m->started || m->fused) return fail(c, ELFEL_ERR_STATE, "assemble!: call start! first (COO mode)");
  if (n < 0 || (n > 0 && (!rows || !cols || !vals))) return fail(c, ELFEL_ERR_ARG, "assemble!: bad arrays");
  if (n == 0) return ELFEL_OK;
  cudaSetDevice(c->device);
  CooStage* s = stage_of(m);
  ELFEL_TRY(ensure_cap(c, &s->I, (size_t)s->n, (size_t)(s->n + n)));
  ELFEL_TRY(ensure_cap(c, &s->J, (size_t)s->n, (size_t)(s->n + n)));
  ELFEL_TRY(ensure_cap(c, &s->V, (size_t)s->n, (size_t)(s->n + n)));
  ELFEL_CUDA(c, cudaMemcpyAsync(s->I.p + s->n, rows, sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(s->J.p + s->n, cols, sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->stream));
  ELFEL_CUDA(c, cudaMemcpyAsync(s->V.p + s->n, vals, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  s->n += n;
  m->finished = 0;
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_finish(elfel_sysmat* m, int64_t* nnz) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (!m->started) return fail(c, ELFEL_ERR_STATE, "finish!: call start! first");
  cudaSetDevice(c->device);
  if (!m->fused) {
    CooStage* s = stage_of(m);
    const int64_t n = s->n;
    DBuf<int32_t> I, J;
    DBuf<int> bad;
    ELFEL_TRY(I.alloc(c, (size_t)(n > 0 ? n : 1)));
    ELFEL_TRY(J.alloc(c, (size_t)(n > 0 ? n : 1)));
    ELFEL_TRY(bad.alloc(c, 1));
    ELFEL_CUDA(c, cudaMemsetAsync(bad.p, 0, sizeof(int), c->stream));
    if (n > 0) {
      const unsigned g = grid_for(n, 256, (int64_t)c->sm_count * 16);
      coo_index_k<<<g, 256, 0, c->stream>>>(s->I.p, n, m->nrow, I.p, bad.p);
      coo_index_k<<<g, 256, 0, c->stream>>>(s->J.p, n, m->ncol, J.p, bad.p);
      ELFEL_LAUNCH_CHECK(c);
    }
    int hbad = 0;
    ELFEL_CUDA(c, cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    bad.release(c);
    if (hbad) {
      I.release(c);
      J.release(c);
      return fail(c, ELFEL_ERR_ARG, "assemble!: row/column number outside 1..%lld / 1..%lld", (long long)m->nrow,
                  (long long)m->ncol);
    }
    SlotGen g;
    g.I = I.p;
    g.J = J.p;
    g.ncoo = n;
    {
      Phase ph(c, "pattern_coo");
      ELFEL_TRY(build_pattern(c, g, m->nrow, m->ncol, &m->P));
      ELFEL_TRY(record_pattern(m));
    }
    I.release(c);
    J.release(c);
    ELFEL_TRY(m->vals.alloc(c, (size_t)(m->P.nnz > 0 ? m->P.nnz : 1)));
    {
      Phase ph(c, "reduce_coo");
      ELFEL_TRY(reduce_values(c, m->P, s->V.p, m->vals.p));
    }
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    m->values_version++;
  }
  m->finished = 1;
  if (nnz) *nnz = m->P.nnz;
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_dims(const elfel_sysmat* m, int64_t* nrow, int64_t* ncol, int64_t* nnz) {
  if (!m) return ELFEL_ERR_ARG;
  if (nrow) *nrow = m->nrow;
  if (ncol) *ncol = m->ncol;
  if (nnz) *nnz = m->P.nnz;
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_csc(elfel_sysmat* m, int64_t* colptr, int64_t* rowval, double* nzval) {
  CHECK_M(m);
  Ctx* c = &m->h->c;
  if (!m->finished) return fail(c, ELFEL_ERR_STATE, "csc: call finish! first");
  cudaSetDevice(c->device);
  const int64_t nnz = m->P.nnz, ncol = m->P.ncol;
  const unsigned grid = grid_for(nnz > ncol + 1 ? nnz : ncol + 1, 256, (int64_t)c->sm_count * 16);
  int pin_c = 0, pin_r = 0;
  int64_t* cpd = colptr ? (int64_t*)host_device_ptr(c, colptr, &pin_c) : nullptr;
  int64_t* rvd = rowval ? (int64_t*)host_device_ptr(c, rowval, &pin_r) : nullptr;
  if (colptr && rowval && cpd && rvd && pin_c && pin_r) {
    // pinned arrays: the 1-based indices are written straight into them (one
    // block per SM: more blocks writing across the host link run slower;
    // pageable arrays take the staged copy, which measured faster there).
    // The indices depend on the pattern only: they go out on the auxiliary
    // stream from the moment the pattern was complete, alongside the values'
    // assembly still running on the context stream, whose copy follows it.
    cudaStream_t s = c->stream;
    if (m->pattern_recorded) ELFEL_TRY(aux_after(c, m->ev_pattern, &s));
    csc_out_k<<<(unsigned)c->sm_count, 256, 0, s>>>(m->P.colptr.p, ncol, m->P.rowval.p, nnz, cpd, rvd);
    ELFEL_LAUNCH_CHECK(c);
    if (nzval && nnz)
      ELFEL_CUDA(c, cudaMemcpyAsync(nzval, m->vals.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, c->stream));
    if (s != c->stream) ELFEL_TRY(aux_join(c));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    return ELFEL_OK;
  }
  DBuf<int64_t> cp, rv;
  ELFEL_TRY(cp.alloc(c, (size_t)ncol + 1));
  ELFEL_TRY(rv.alloc(c, (size_t)(nnz > 0 ? nnz : 1)));
  csc_out_k<<<grid, 256, 0, c->stream>>>(m->P.colptr.p, ncol, m->P.rowval.p, nnz, cp.p, rv.p);
  ELFEL_LAUNCH_CHECK(c);
  if (colptr) ELFEL_CUDA(c, cudaMemcpyAsync(colptr, cp.p, sizeof(int64_t) * (ncol + 1), cudaMemcpyDeviceToHost, c->stream));
  if (rowval && nnz)
    ELFEL_CUDA(c, cudaMemcpyAsync(rowval, rv.p, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, c->stream));
  if (nzval && nnz)
    ELFEL_CUDA(c, cudaMemcpyAsync(nzval, m->vals.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, c->stream));
  cp.release(c);
  rv.release(c);
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_rhs(elfel_sysmat* m, double* F) {
  CHECK_M(m);
  Ctx* c = &m->h->c;
  if (!m->has_rhs) return fail(c, ELFEL_ERR_STATE, "rhs: no fused assembly has run");
  cudaSetDevice(c->device);
  if (F && m->nrow)
    ELFEL_CUDA(c, cudaMemcpyAsync(F, m->rhs.p, sizeof(double) * m->nrow, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  return ELFEL_OK;
}

extern "C" int elfel_sysvec_assemble(elfel_ctx* h, int64_t nrow, const int64_t* rows, const double* vals, int64_t n,
                                     double* out) {
  if (!h) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  if (nrow < 0 || n < 0 || (n > 0 && (!rows || !vals)) || (nrow > 0 && !out))
    return fail(c, ELFEL_ERR_ARG, "sysvec: bad arguments");
  cudaSetDevice(c->device);
  DBuf<int32_t> J;
  DBuf<double> V, dense;
  ELFEL_TRY(to_index32(c, rows, n, nrow, &J, "SysvecAssembler row"));
  ELFEL_TRY(V.alloc(c, (size_t)(n > 0 ? n : 1)));
  if (n) ELFEL_CUDA(c, cudaMemcpyAsync(V.p, vals, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  SlotGen g;
  g.nel = n;
  g.slots_per_elem = 1;
  g.store_per_elem = 1;
  g.nblocks = 1;
  g.b[0].R = nullptr;
  g.b[0].C = J.p;
  g.b[0].nr = 1;
  g.b[0].nc = 1;
  Pattern P;
  ELFEL_TRY(build_pattern(c, g, 1, nrow, &P));
  ELFEL_TRY(dense.alloc(c, (size_t)(nrow > 0 ? nrow : 1)));
  ELFEL_TRY(reduce_dense(c, P, V.p, dense.p));
  if (nrow) ELFEL_CUDA(c, cudaMemcpyAsync(out, dense.p, sizeof(double) * nrow, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  P.release(c);
  J.release(c);
  V.release(c);
  dense.release(c);
  return ELFEL_OK;
}

// ------------------------------------------------------------------ fused
static int upload_space(Ctx* c, const elfel_space& s, int64_t ndofs, int sdim, DBuf<int32_t>* conn,
                        DBuf<double>* xy, DBuf<int32_t>* dofs, const char* name) {
  if (s.nel < 0 || s.nnodes < 0 || !s.conn || !s.eldofs || (s.nnodes > 0 && !s.xy))
    return fail(c, ELFEL_ERR_ARG, "%s space: missing arrays", name);
  const int nedof = s.nodes_per_elem * s.ncomp;
  std::string w1 = std::string(name) + " connectivity";
  std::string w2 = std::string(name) + " eldofs";
  ELFEL_TRY(to_index32(c, s.conn, s.nel * s.nodes_per_elem, s.nnodes, conn, w1.c_str()));
  ELFEL_TRY(to_index32(c, s.eldofs, s.nel * nedof, ndofs, dofs, w2.c_str()));
  if (xy) {
    ELFEL_TRY(xy->alloc(c, (size_t)(s.nnodes > 0 ? sdim * s.nnodes : 1)));
    if (s.nnodes)
      ELFEL_CUDA(c, cudaMemcpyAsync(xy->p, s.xy, sizeof(double) * sdim * s.nnodes, cudaMemcpyHostToDevice,
                                    c->stream));
  }
  return ELFEL_OK;
}

// Upload of the mesh tables when every host array is device-readable
// (host_device_ptr): the element DOFs, which the pattern build reads, on the
// context stream; connectivity and coordinates on the auxiliary stream, so
// that they cross the host link while the pattern is built (fused_build joins
// before it uses them).  The index checks are deferred: bad[0..3] (primary
// connectivity, primary DOFs, pressure connectivity, pressure DOFs) are read
// once the work of both streams is done.
static bool tables_readable(Ctx* c, const elfel_space& s) {
  if (s.nel < 0 || s.nnodes < 0 || !s.conn || !s.eldofs || (s.nnodes > 0 && !s.xy))
    return false;  // upload_space reports the error
  return (s.nel == 0 || (host_device_ptr(c, s.conn) && host_device_ptr(c, s.eldofs))) &&
         (s.nnodes == 0 || host_device_ptr(c, s.xy));
}

// Step 1 (context stream): the buffers, then the element DOFs.
static int upload_direct_dofs(Ctx* c, const elfel_space& s, int64_t ndofs, int sdim, DBuf<int32_t>* conn,
                              DBuf<double>* xy, DBuf<int32_t>* dofs, int* bad_dofs) {
  const int64_t nc = s.nel * s.nodes_per_elem, nd = s.nel * s.nodes_per_elem * s.ncomp;
  ELFEL_TRY(conn->alloc(c, (size_t)(nc > 0 ? nc : 1)));
  ELFEL_TRY(dofs->alloc(c, (size_t)(nd > 0 ? nd : 1)));
  if (xy) ELFEL_TRY(xy->alloc(c, (size_t)(s.nnodes > 0 ? sdim * s.nnodes : 1)));
  return to_index32_direct(c, c->stream, (const int64_t*)host_device_ptr(c, s.eldofs), nd, ndofs, dofs->p,
                           bad_dofs);
}

// Step 2 (auxiliary stream, forked after step 1's allocations): connectivity
// and coordinates.
static int upload_direct_rest(Ctx* c, const elfel_space& s, int sdim, DBuf<int32_t>* conn, DBuf<double>* xy,
                              int* bad_conn, cudaStream_t aux) {
  ELFEL_TRY(to_index32_direct(c, aux, (const int64_t*)host_device_ptr(c, s.conn), s.nel * s.nodes_per_elem,
                              s.nnodes, conn->p, bad_conn));
  if (xy && s.nnodes) {
    int pinned = 0;
    const double* src = (const double*)host_device_ptr(c, s.xy, &pinned);
    ELFEL_TRY(copy_host_f64(c, aux, pinned ? s.xy : src, pinned, sdim * s.nnodes, xy->p));
  }
  return ELFEL_OK;
}

// The checks of a fused descriptor shared by both set-ups (the element DOF
// tables are checked where they are read).
static int check_fused_desc(Ctx* c, const elfel_fused_desc* d) {
  if (!d) return fail(c, ELFEL_ERR_ARG, "fused_setup: NULL descriptor");
  if (d->ndofs < 0) return fail(c, ELFEL_ERR_ARG, "fused_setup: negative ndofs");
  const elfel_space& u = d->u;
  const int sdim = d->sdim ? d->sdim : 2;
  if (d->shape == ELFEL_SHAPE_TRIANGLE) {
    if (u.nodes_per_elem != 3 && u.nodes_per_elem != 6)
      return fail(c, ELFEL_ERR_UNSUPPORTED, "fused_setup: triangles with %d nodes are not provided (T3, T6 only)",
                  u.nodes_per_elem);
  } else if (d->shape == ELFEL_SHAPE_Q4 || d->shape == ELFEL_SHAPE_T4) {
    if (u.nodes_per_elem != 4)
      return fail(c, ELFEL_ERR_ARG, "fused_setup: %s elements have 4 nodes (got %d)",
                  d->shape == ELFEL_SHAPE_Q4 ? "Q4" : "T4", u.nodes_per_elem);
    if (d->physics != ELFEL_HEAT)
      return fail(c, ELFEL_ERR_UNSUPPORTED, "fused_setup: Q4 and T4 elements take the heat weak form only");
  } else {
    return fail(c, ELFEL_ERR_ARG, "fused_setup: unknown element shape %d", d->shape);
  }
  if (sdim != (d->shape == ELFEL_SHAPE_T4 ? 3 : 2))
    return fail(c, ELFEL_ERR_ARG, "fused_setup: %d coordinates per node for this element shape", sdim);
  if (d->npts < 1 || d->npts > kMaxQP || !d->qp_coords || !d->qp_weights)
    return fail(c, ELFEL_ERR_ARG, "fused_setup: quadrature with %d points (1..%d)", d->npts, kMaxQP);
  if (d->physics == ELFEL_HEAT && u.ncomp != 1)
    return fail(c, ELFEL_ERR_ARG, "heat: scalar space expected (ncomp = %d)", u.ncomp);
  if (d->physics == ELFEL_ELASTICITY && u.ncomp != 2)
    return fail(c, ELFEL_ERR_ARG, "elasticity: 2-component space expected (ncomp = %d)", u.ncomp);
  if (d->physics == ELFEL_STOKES) {
    if (u.nodes_per_elem != 6 || u.ncomp != 2 || d->p.nodes_per_elem != 3 || d->p.ncomp != 1 || d->p.nel != u.nel)
      return fail(c, ELFEL_ERR_UNSUPPORTED, "Stokes: vector T6 velocity and scalar T3 pressure on the same elements");
  } else if (d->physics != ELFEL_HEAT && d->physics != ELFEL_ELASTICITY) {
    return fail(c, ELFEL_ERR_ARG, "fused_setup: unknown physics %d", d->physics);
  }
  return ELFEL_OK;
}

// Releases the system's buffers and records the descriptor's sizes and tables.
static int init_fused(elfel_sysmat* m, const elfel_fused_desc* d) {
  Ctx* c = &m->h->c;
  const elfel_space& u = d->u;
  release_all(m);
  Fused& F = m->F;
  F.physics = d->physics;
  F.npts = d->npts;
  F.shape = d->shape;
  F.sdim = d->sdim ? d->sdim : 2;
  F.nn_u = u.nodes_per_elem;
  F.ncomp_u = u.ncomp;
  F.nel = u.nel;
  F.nnodes_u = u.nnodes;
  if (F.shape == ELFEL_SHAPE_TRIANGLE)
    ELFEL_TRY(make_tables(u.nodes_per_elem, d->npts, d->qp_coords, d->qp_weights, &F.tab));
  else
    ELFEL_TRY(make_shape_tables(F.shape, d->npts, d->qp_coords, d->qp_weights, &F.stab));
  if (d->physics == ELFEL_STOKES) {
    F.nn_p = 3;
    F.nnodes_p = d->p.nnodes;
  }
  return ELFEL_OK;
}

extern "C" int elfel_fused_setup(elfel_sysmat* m, const elfel_fused_desc* d) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  cudaSetDevice(c->device);
  ELFEL_TRY(check_fused_desc(c, d));
  const elfel_space& u = d->u;
  const int sdim = d->sdim ? d->sdim : 2;
  ELFEL_TRY(init_fused(m, d));
  Fused& F = m->F;
  const bool stokes = d->physics == ELFEL_STOKES;
  if (!tables_readable(c, u) || (stokes && !tables_readable(c, d->p))) {
    ELFEL_TRY(upload_space(c, u, d->ndofs, sdim, &F.conn_u, &F.xy_u, &F.dofs_u, "primary"));
    if (stokes) ELFEL_TRY(upload_space(c, d->p, d->ndofs, 2, &F.conn_p, nullptr, &F.dofs_p, "pressure"));
    return fused_build(m, d->ndofs);
  }
  DBuf<int> bad;
  auto run = [&]() -> int {
    ELFEL_TRY(bad.alloc(c, 4));
    ELFEL_CUDA(c, cudaMemsetAsync(bad.p, 0, 4 * sizeof(int), c->stream));
    ELFEL_TRY(upload_direct_dofs(c, u, d->ndofs, sdim, &F.conn_u, &F.xy_u, &F.dofs_u, bad.p + 1));
    if (stokes) ELFEL_TRY(upload_direct_dofs(c, d->p, d->ndofs, 2, &F.conn_p, nullptr, &F.dofs_p, bad.p + 3));
    cudaStream_t aux;
    ELFEL_TRY(aux_fork(c, &aux));  // after the allocations, which the auxiliary stream then may use
    ELFEL_TRY(upload_direct_rest(c, u, sdim, &F.conn_u, &F.xy_u, bad.p, aux));
    if (stokes) ELFEL_TRY(upload_direct_rest(c, d->p, 2, &F.conn_p, nullptr, bad.p + 2, aux));
    ELFEL_TRY(fused_build(m, d->ndofs));  // joins the auxiliary stream before using conn / xy
    int hb[4] = {0, 0, 0, 0};
    ELFEL_CUDA(c, cudaMemcpyAsync(hb, bad.p, sizeof(hb), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    static const char* what[4] = {"primary connectivity", "primary eldofs", "pressure connectivity",
                                  "pressure eldofs"};
    const int64_t lim[4] = {u.nnodes, d->ndofs, stokes ? d->p.nnodes : 0, d->ndofs};
    for (int k = 0; k < 4; ++k)
      if (hb[k]) return fail(c, ELFEL_ERR_ARG, "%s: entry outside 1..%lld", what[k], (long long)lim[k]);
    return ELFEL_OK;
  };
  const int rc = run();
  if (rc != ELFEL_OK) {
    aux_join(c);
    cudaStreamSynchronize(c->stream);
    release_all(m);
  }
  bad.release(c);
  return rc;
}

namespace elfel {

// Slot generators, patterns and value buffers of a fused system whose tables
// (connectivity, coordinates, element DOFs) are already on the device.
int fused_build(elfel_sysmat* m, int64_t ndofs) {
  Ctx* c = &m->h->c;
  Fused& F = m->F;
  const int nedof = F.nn_u * F.ncomp_u;
  SlotGen& g = F.kgen;
  g = SlotGen();
  g.nel = F.nel;
  g.nblocks = 1;
  g.b[0].R = F.dofs_u.p;
  g.b[0].C = F.dofs_u.p;
  g.b[0].nr = g.b[0].nc = nedof;
  g.b[0].sym = 1;
  g.slots_per_elem = nedof * nedof;
  g.store_per_elem = nedof * (nedof + 1) / 2;
  if (F.physics == ELFEL_STOKES) {
    g.nblocks = 3;
    g.b[1].R = F.dofs_u.p;
    g.b[1].C = F.dofs_p.p;
    g.b[1].nr = 12;
    g.b[1].nc = 3;
    g.b[1].slot_off = 144;
    g.b[1].store_off = 78;
    g.b[2] = g.b[1];
    g.b[2].transposed = 1;
    g.b[2].slot_off = 180;
    g.slots_per_elem = 216;
    g.store_per_elem = 78 + 36;
  }
  m->nrow = m->ncol = ndofs;
  {
    Phase ph(c, "pattern_K");
    ELFEL_TRY(build_pattern(c, g, ndofs, ndofs, &m->P));
    ELFEL_TRY(record_pattern(m));
  }
  // right-hand side: a 1 x ndofs "matrix" of the element vectors
  SlotGen& fg = F.fgen;
  fg = SlotGen();
  fg.nel = F.nel;
  fg.nblocks = 1;
  fg.b[0].R = nullptr;
  fg.b[0].C = F.dofs_u.p;
  fg.b[0].nr = 1;
  fg.b[0].nc = nedof;
  fg.slots_per_elem = nedof;
  fg.store_per_elem = nedof;
  F.fpat_built = 0;  // built on first use (ensure_fpat)
  if (F.physics == ELFEL_STOKES) {
    SlotGen pg;
    pg.nel = F.nel;
    pg.nblocks = 1;
    pg.b[0].R = nullptr;
    pg.b[0].C = F.dofs_p.p;
    pg.b[0].nr = 1;
    pg.b[0].nc = 3;
    pg.slots_per_elem = 3;
    pg.store_per_elem = 3;
    ELFEL_TRY(build_pattern(c, pg, 1, ndofs, &F.pmpat));
    ELFEL_TRY(F.pmass_store.alloc(c, (size_t)(F.nel * 3 > 0 ? F.nel * 3 : 1)));
    ELFEL_TRY(F.pmass_diag.alloc(c, (size_t)(ndofs > 0 ? ndofs : 1)));
  }
  ELFEL_TRY(aux_join(c));  // tables uploaded on the auxiliary stream
  F.f_direct_ok = 0;
  if (F.physics == ELFEL_HEAT && F.shape == ELFEL_SHAPE_TRIANGLE && F.nn_u == 6 && F.ncomp_u == 1 && F.nel > 0) {
    // the T6 load vector may be added atomically (launch_heat) when no DOF
    // collects more than two nonzero element contributions
    DBuf<int32_t> cnt;  // ndofs counters, then the flag
    int h_many = 1;
    auto count = [&]() -> int {
      ELFEL_TRY(cnt.alloc(c, (size_t)ndofs + 1));
      ELFEL_CUDA(c, cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (ndofs + 1), c->stream));
      midside_count_k<<<grid_for(F.nel * 3, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(
          F.dofs_u.p, F.nel, cnt.p, cnt.p + ndofs);
      ELFEL_LAUNCH_CHECK(c);
      ELFEL_CUDA(c, cudaMemcpyAsync(&h_many, cnt.p + ndofs, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
      return ELFEL_OK;
    };
    const int rc = count();
    cnt.release(c);
    if (rc != ELFEL_OK) return rc;
    F.f_direct_ok = h_many == 0;
  }
  ELFEL_TRY(F.straight.alloc(c, (size_t)(F.nel > 0 ? F.nel : 1)));
  if (F.shape == ELFEL_SHAPE_TRIANGLE)
    ELFEL_TRY(launch_straight(c, F.nn_u, F.nel, F.conn_u.p, F.xy_u.p, F.straight.p, &F.ncurved));
  ELFEL_TRY(F.kstore.alloc(c, (size_t)(F.nel * g.store_per_elem > 0 ? F.nel * g.store_per_elem : 1)));
  ELFEL_TRY(F.fstore.alloc(c, (size_t)(F.nel * nedof > 0 ? F.nel * nedof : 1)));
  ELFEL_TRY(m->vals.alloc(c, (size_t)(m->P.nnz > 0 ? m->P.nnz : 1)));
  ELFEL_TRY(m->rhs.alloc(c, (size_t)(ndofs > 0 ? ndofs : 1)));
  ELFEL_TRY(F.coef.alloc(c, (size_t)(F.nel > 0 ? 2 * F.nel : 1)));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  m->fused = 1;
  m->started = 1;
  m->finished = 0;
  return ELFEL_OK;
}

}  // namespace elfel

extern "C" int elfel_fused_setup_block(elfel_sysmat* m, const elfel_block_desc* d, int64_t* ndofs, int64_t* nu) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (!d) return fail(c, ELFEL_ERR_ARG, "setup_block: NULL descriptor");
  if (d->npts < 1 || d->npts > kMaxQP || !d->qp_coords || !d->qp_weights)
    return fail(c, ELFEL_ERR_ARG, "setup_block: quadrature with %d points (1..%d)", d->npts, kMaxQP);
  if (d->nodes_per_elem != 3 && d->nodes_per_elem != 6)
    return fail(c, ELFEL_ERR_UNSUPPORTED, "setup_block: T3 or T6 blocks (nodes_per_elem %d)", d->nodes_per_elem);
  cudaSetDevice(c->device);
  release_all(m);
  Fused& F = m->F;
  F.physics = ELFEL_HEAT;
  F.npts = d->npts;
  ELFEL_TRY(make_tables(d->nodes_per_elem, d->npts, d->qp_coords, d->qp_weights, &F.tab));
  int64_t nfree = 0;
  ELFEL_TRY(block_tables(c, *d, &F, &nfree));
  F.is_block = 1;
  F.block = *d;
  F.block.qp_coords = nullptr;  // not kept
  F.block.qp_weights = nullptr;
  ELFEL_TRY(fused_build(m, F.nnodes_u));
  if (ndofs) *ndofs = F.nnodes_u;
  if (nu) *nu = nfree;
  return ELFEL_OK;
}

extern "C" int elfel_number_dofs(elfel_ctx* h, int32_t nspaces, const int64_t* nterms, const int32_t* ncomp,
                                 const uint8_t* const* isdatum, int64_t* const* dofnums, int64_t* nfree) {
  if (!h) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  if (nspaces < 1 || nspaces > 64 || !nterms || !ncomp || !isdatum)
    return fail(c, ELFEL_ERR_ARG, "number_dofs: %d spaces", (int)nspaces);
  cudaSetDevice(c->device);
  std::vector<int64_t> n(nspaces);
  int64_t total = 0;
  for (int s = 0; s < nspaces; ++s) {
    if (nterms[s] < 0 || ncomp[s] < 1 || (nterms[s] > 0 && !isdatum[s]))
      return fail(c, ELFEL_ERR_ARG, "number_dofs: space %d: %lld terms of %d components", s, (long long)nterms[s],
                  (int)ncomp[s]);
    n[s] = nterms[s] * ncomp[s];
    total += n[s];
  }
  if (total >= 0x7fffffff) return fail(c, ELFEL_ERR_ARG, "number_dofs: %lld DOFs (at most 2^31 - 1)", (long long)total);
  std::vector<DBuf<uint8_t>> mk(nspaces);
  std::vector<DBuf<int32_t>> nm(nspaces);
  auto run = [&]() -> int {
    std::vector<const uint8_t*> masks(nspaces);
    std::vector<int32_t*> nums(nspaces);
    for (int s = 0; s < nspaces; ++s) {
      ELFEL_TRY(mk[s].alloc(c, (size_t)(n[s] > 0 ? n[s] : 1)));
      ELFEL_TRY(nm[s].alloc(c, (size_t)(n[s] > 0 ? n[s] : 1)));
      if (n[s]) ELFEL_CUDA(c, cudaMemcpyAsync(mk[s].p, isdatum[s], n[s], cudaMemcpyHostToDevice, c->stream));
      masks[s] = mk[s].p;
      nums[s] = nm[s].p;
    }
    ELFEL_TRY(number_spaces(c, nspaces, masks.data(), n.data(), nums.data(), nfree));
    for (int s = 0; s < nspaces; ++s)
      if (dofnums && dofnums[s]) ELFEL_TRY(numbers_to_host(c, nm[s].p, n[s], dofnums[s]));
    return ELFEL_OK;
  };
  const int rc = run();
  for (int s = 0; s < nspaces; ++s) {
    mk[s].release(c);
    nm[s].release(c);
  }
  return rc;
}

extern "C" int elfel_fused_setup_numbered(elfel_sysmat* m, const elfel_fused_desc* d, const uint8_t* isdatum_u,
                                          const uint8_t* isdatum_p, int64_t* dofnums_u, int64_t* dofnums_p,
                                          int64_t* nfree) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  cudaSetDevice(c->device);
  ELFEL_TRY(check_fused_desc(c, d));
  const bool stokes = d->physics == ELFEL_STOKES;
  const elfel_space& u = d->u;
  const int sdim = d->sdim ? d->sdim : 2;
  const int64_t nu_terms = u.nnodes * u.ncomp, np_terms = stokes ? d->p.nnodes : 0;
  if (!isdatum_u || (stokes && !isdatum_p))
    return fail(c, ELFEL_ERR_ARG, "fused_setup_numbered: NULL essential-BC mask");
  if (u.nel < 0 || u.nnodes < 0 || !u.conn || (u.nnodes > 0 && !u.xy) || (stokes && !d->p.conn))
    return fail(c, ELFEL_ERR_ARG, "fused_setup_numbered: missing connectivity or coordinates");
  if (d->ndofs != nu_terms + np_terms)
    return fail(c, ELFEL_ERR_ARG, "fused_setup_numbered: ndofs %lld, the spaces hold %lld DOFs",
                (long long)d->ndofs, (long long)(nu_terms + np_terms));
  ELFEL_TRY(init_fused(m, d));
  Fused& F = m->F;
  DBuf<uint8_t> mu, mp;
  DBuf<int32_t> nu_, np_;
  auto run = [&]() -> int {
    ELFEL_TRY(to_index32(c, u.conn, u.nel * u.nodes_per_elem, u.nnodes, &F.conn_u, "primary connectivity"));
    ELFEL_TRY(F.xy_u.alloc(c, (size_t)(u.nnodes > 0 ? sdim * u.nnodes : 1)));
    if (u.nnodes)
      ELFEL_CUDA(c, cudaMemcpyAsync(F.xy_u.p, u.xy, sizeof(double) * sdim * u.nnodes, cudaMemcpyHostToDevice,
                                    c->stream));
    if (stokes)
      ELFEL_TRY(to_index32(c, d->p.conn, d->p.nel * 3, d->p.nnodes, &F.conn_p, "pressure connectivity"));
    ELFEL_TRY(mu.alloc(c, (size_t)(nu_terms > 0 ? nu_terms : 1)));
    ELFEL_TRY(nu_.alloc(c, (size_t)(nu_terms > 0 ? nu_terms : 1)));
    if (nu_terms)
      ELFEL_CUDA(c, cudaMemcpyAsync(mu.p, isdatum_u, nu_terms, cudaMemcpyHostToDevice, c->stream));
    if (stokes) {
      ELFEL_TRY(mp.alloc(c, (size_t)(np_terms > 0 ? np_terms : 1)));
      ELFEL_TRY(np_.alloc(c, (size_t)(np_terms > 0 ? np_terms : 1)));
      if (np_terms)
        ELFEL_CUDA(c, cudaMemcpyAsync(mp.p, isdatum_p, np_terms, cudaMemcpyHostToDevice, c->stream));
    }
    const uint8_t* masks[2] = {mu.p, mp.p};
    const int64_t ns[2] = {nu_terms, np_terms};
    int32_t* nums[2] = {nu_.p, np_.p};
    int64_t nf = 0;
    ELFEL_TRY(number_spaces(c, stokes ? 2 : 1, masks, ns, nums, &nf));
    const int nedof_u = u.nodes_per_elem * u.ncomp;
    ELFEL_TRY(F.dofs_u.alloc(c, (size_t)(u.nel * nedof_u > 0 ? u.nel * nedof_u : 1)));
    ELFEL_TRY(element_dofs(c, F.conn_u.p, u.nel, u.nodes_per_elem, u.ncomp, nu_.p, F.dofs_u.p));
    if (stokes) {
      ELFEL_TRY(F.dofs_p.alloc(c, (size_t)(d->p.nel * 3 > 0 ? d->p.nel * 3 : 1)));
      ELFEL_TRY(element_dofs(c, F.conn_p.p, d->p.nel, 3, 1, np_.p, F.dofs_p.p));
    }
    ELFEL_TRY(numbers_to_host(c, nu_.p, nu_terms, dofnums_u));
    if (stokes) ELFEL_TRY(numbers_to_host(c, np_.p, np_terms, dofnums_p));
    if (nfree) *nfree = nf;
    return fused_build(m, d->ndofs);
  };
  const int rc = run();
  mu.release(c);
  mp.release(c);
  nu_.release(c);
  np_.release(c);
  if (rc != ELFEL_OK) {
    cudaStreamSynchronize(c->stream);
    release_all(m);
  }
  return rc;
}

extern "C" int elfel_block_dirichlet(elfel_sysmat* m, const double* coef6, double* T) {
  CHECK_M(m);
  Ctx* c = &m->h->c;
  if (!m->fused || !m->F.is_block) return fail(c, ELFEL_ERR_STATE, "block_dirichlet: not a block system");
  if (!coef6 || !T) return fail(c, ELFEL_ERR_ARG, "block_dirichlet: NULL argument");
  cudaSetDevice(c->device);
  const int64_t n = m->F.nnodes_u;
  DBuf<double> d;
  ELFEL_TRY(d.alloc(c, (size_t)n));
  ELFEL_TRY(block_dirichlet(c, m->F.block, coef6, m->F, d.p));
  ELFEL_CUDA(c, cudaMemcpyAsync(T, d.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  d.release(c);
  return ELFEL_OK;
}

extern "C" int elfel_fused_tables(elfel_sysmat* m, int64_t* conn, double* xy, int64_t* eldofs) {
  CHECK_M(m);
  Ctx* c = &m->h->c;
  if (!m->fused) return fail(c, ELFEL_ERR_STATE, "fused_tables: not a fused system");
  cudaSetDevice(c->device);
  return tables_to_host(c, m->F, conn, xy, eldofs);
}

extern "C" int elfel_fused_dims(elfel_sysmat* m, int64_t* nel, int64_t* nnodes, int64_t* ndofs) {
  CHECK_M(m);
  if (!m->fused) return fail(&m->h->c, ELFEL_ERR_STATE, "fused_dims: not a fused system");
  if (nel) *nel = m->F.nel;
  if (nnodes) *nnodes = m->F.nnodes_u;
  if (ndofs) *ndofs = m->nrow;
  return ELFEL_OK;
}

extern "C" int elfel_sysmat_tile_stats(elfel_sysmat* m, int64_t* ntiles, int64_t* nprograms, int64_t* nfallback,
                                       int64_t* nruns) {
  CHECK_M(m);
  const TilePlan& T = m->P.tiles;
  if (ntiles) *ntiles = T.built ? T.ntiles : 0;
  if (nprograms) *nprograms = T.built ? T.nprograms : 0;
  if (nfallback) *nfallback = T.built ? T.nfallback : 0;
  if (nruns) *nruns = T.built ? T.nruns : 0;
  return ELFEL_OK;
}

extern "C" int elfel_fused_set_geometry(elfel_sysmat* m, const double* xy) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (!m->fused) return fail(c, ELFEL_ERR_STATE, "set_geometry: call fused_setup first");
  if (!xy) return fail(c, ELFEL_ERR_ARG, "set_geometry: NULL coordinates");
  cudaSetDevice(c->device);
  if (m->F.nnodes_u)
    ELFEL_CUDA(c, cudaMemcpyAsync(m->F.xy_u.p, xy, sizeof(double) * m->F.sdim * m->F.nnodes_u,
                                  cudaMemcpyHostToDevice, c->stream));
  if (m->F.shape != ELFEL_SHAPE_TRIANGLE) return ELFEL_OK;
  return launch_straight(c, m->F.nn_u, m->F.nel, m->F.conn_u.p, m->F.xy_u.p, m->F.straight.p, &m->F.ncurved);
}

int elfel::ensure_fpat(elfel_sysmat* m) {
  Fused& F = m->F;
  if (F.fpat_built) return ELFEL_OK;
  Ctx* c = &m->h->c;
  Phase ph(c, "pattern_F");
  ELFEL_TRY(build_pattern(c, F.fgen, 1, m->ncol, &F.fpat));
  F.fpat_built = 1;
  return ELFEL_OK;
}

// rhs_done: the integration kernel already added the load vector into rhs.
static int finish_values(elfel_sysmat* m, bool rhs_done = false) {
  Ctx* c = &m->h->c;
  {
    Phase ph(c, "reduce_K");
    ELFEL_TRY(reduce_values(c, m->P, m->F.kstore.p, m->vals.p));
  }
  if (!rhs_done) {
    ELFEL_TRY(ensure_fpat(m));
    Phase ph(c, "reduce_F");
    ELFEL_TRY(reduce_dense(c, m->F.fpat, m->F.fstore.p, m->rhs.p));
  }
  m->has_rhs = 1;
  m->finished = 1;
  m->values_version++;
  return ELFEL_OK;
}

extern "C" int elfel_fused_heat(elfel_sysmat* m, const double* kappa, double Q) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (!m->fused || m->F.physics != ELFEL_HEAT) return fail(c, ELFEL_ERR_STATE, "heat: fused_setup(ELFEL_HEAT) first");
  cudaSetDevice(c->device);
  Fused& F = m->F;
  if (kappa && F.nel)
    ELFEL_CUDA(c, cudaMemcpyAsync(F.coef.p, kappa, sizeof(double) * F.nel, cudaMemcpyHostToDevice, c->stream));
  const bool fdirect = F.shape == ELFEL_SHAPE_TRIANGLE && F.f_direct_ok && heat_f_direct(F.nn_u, F.ncurved, F.tab);
  // From a pattern's second assembly on, an exact-rule straight-sided T6 mesh
  // writes 8 bases per element and the tile reduction expands and sums them
  // (the plan is built once, at that assembly); a pattern assembled once (an
  // end-to-end call) keeps the records and the contributor-list reduction.
  // Both give the same bits.
  const bool tiles = c->tiles && F.shape == ELFEL_SHAPE_TRIANGLE && heat_bases_ok(F.nn_u, F.ncurved, F.tab) &&
                     m->P.reductions >= 1 && m->P.nslots < 0x7fffffff;
  if (tiles) {
    if (!(m->P.tiles.built && m->P.tiles.V == kT6RTable && m->P.tiles.S == 21)) {
      Phase ph(c, "tile_plan");
      ELFEL_TRY(build_tile_plan(c, m->P, 21, kT6RTable, kT6REntry));
    }
    {
      Phase ph(c, "integrate_heat");
      if (fdirect) ELFEL_CUDA(c, cudaMemsetAsync(m->rhs.p, 0, sizeof(double) * m->ncol, c->stream));
      ELFEL_TRY(launch_heat_bases(c, F.nel, F.conn_u.p, F.xy_u.p, F.coef.p, Q, F.tab, F.kstore.p, F.fstore.p,
                                  fdirect ? F.dofs_u.p : nullptr, fdirect ? m->rhs.p : nullptr));
    }
    {
      Phase ph(c, "reduce_K");
      ELFEL_TRY(tile_reduce(c, m->P, F.kstore.p, 1, m->vals.p));
    }
    m->P.reductions++;
    if (!fdirect) {
      ELFEL_TRY(ensure_fpat(m));
      Phase ph(c, "reduce_F");
      ELFEL_TRY(reduce_dense(c, m->F.fpat, m->F.fstore.p, m->rhs.p));
    }
    m->has_rhs = 1;
    m->finished = 1;
    m->values_version++;
    return ELFEL_OK;
  }
  {
    Phase ph(c, "integrate_heat");
    if (fdirect) {
      ELFEL_CUDA(c, cudaMemsetAsync(m->rhs.p, 0, sizeof(double) * m->ncol, c->stream));
      ELFEL_TRY(launch_heat(c, F.nn_u, F.nel, F.conn_u.p, F.xy_u.p, F.coef.p, Q, F.straight.p, F.ncurved, F.tab,
                            F.kstore.p, F.fstore.p, F.dofs_u.p, m->rhs.p));
    } else if (F.shape == ELFEL_SHAPE_TRIANGLE) {
      ELFEL_TRY(launch_heat(c, F.nn_u, F.nel, F.conn_u.p, F.xy_u.p, F.coef.p, Q, F.straight.p, F.ncurved, F.tab,
                            F.kstore.p, F.fstore.p));
    } else {
      ELFEL_TRY(launch_heat_shape(c, F.stab, F.nel, F.conn_u.p, F.xy_u.p, F.coef.p, Q, F.kstore.p, F.fstore.p));
    }
  }
  return finish_values(m, fdirect);
}

extern "C" int elfel_fused_elasticity(elfel_sysmat* m, double E, double nu, int32_t plane_strain,
                                      const double* bforce, const int64_t* trac_edges, int64_t ntrac,
                                      const double* traction) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (!m->fused || m->F.physics != ELFEL_ELASTICITY)
    return fail(c, ELFEL_ERR_STATE, "elasticity: fused_setup(ELFEL_ELASTICITY) first");
  if (ntrac < 0 || (ntrac > 0 && (!trac_edges || !traction))) return fail(c, ELFEL_ERR_ARG, "elasticity: traction");
  cudaSetDevice(c->device);
  Fused& F = m->F;
  Mat3 D;
  memset(&D, 0, sizeof(D));
  if (plane_strain) {
    const double f = E / ((1 + nu) * (1 - 2 * nu));
    D.a[0][0] = D.a[1][1] = f * (1 - nu);
    D.a[0][1] = D.a[1][0] = f * nu;
    D.a[2][2] = f * (1 - 2 * nu) / 2;
  } else {
    const double f = E / (1 - nu * nu);
    D.a[0][0] = D.a[1][1] = f;
    D.a[0][1] = D.a[1][0] = f * nu;
    D.a[2][2] = f * (1 - nu) / 2;
  }
  const double* bf = nullptr;
  if (bforce && F.nel) {
    ELFEL_CUDA(c, cudaMemcpyAsync(F.coef.p, bforce, sizeof(double) * 2 * F.nel, cudaMemcpyHostToDevice, c->stream));
    bf = F.coef.p;
  }
  {
    Phase ph(c, "integrate_elasticity");
    ELFEL_TRY(launch_elasticity(c, F.nn_u, F.nel, F.conn_u.p, F.xy_u.p, D, bf, F.ncurved, F.tab, F.kstore.p,
                                F.fstore.p));
  }
  ELFEL_TRY(finish_values(m));
  if (ntrac > 0) {
    const int nen = F.nn_u == 6 ? 3 : 2;
    // (element, local edge) 1-based -> 0-based, range checked
    std::vector<int64_t> flat((size_t)ntrac * 2);
    for (int64_t k = 0; k < ntrac; ++k) {
      int64_t e = trac_edges[2 * k], le = trac_edges[2 * k + 1];
      if (e < 1 || e > F.nel || le < 1 || le > 3) return fail(c, ELFEL_ERR_ARG, "traction edge %lld invalid", (long long)k);
      flat[2 * k] = e;
      flat[2 * k + 1] = le;
    }
    DBuf<int32_t> edges, edofs;
    DBuf<double> tstore, tvec;
    ELFEL_TRY(to_index32(c, flat.data(), 2 * ntrac, F.nel, &edges, "traction edges"));
    ELFEL_TRY(edofs.alloc(c, (size_t)ntrac * nen * 2));
    edge_dofs_k<<<grid_for(ntrac, 128), 128, 0, c->stream>>>(ntrac, edges.p, F.dofs_u.p, F.nn_u, 2, edofs.p);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_TRY(tstore.alloc(c, (size_t)ntrac * nen * 2));
    ELFEL_TRY(launch_traction(c, ntrac, edges.p, F.conn_u.p, F.nn_u, F.xy_u.p, traction[0], traction[1], tstore.p));
    SlotGen tg;
    tg.nel = ntrac;
    tg.nblocks = 1;
    tg.b[0].R = nullptr;
    tg.b[0].C = edofs.p;
    tg.b[0].nr = 1;
    tg.b[0].nc = nen * 2;
    tg.slots_per_elem = nen * 2;
    tg.store_per_elem = nen * 2;
    Pattern tp;
    ELFEL_TRY(build_pattern(c, tg, 1, m->nrow, &tp));
    ELFEL_TRY(tvec.alloc(c, (size_t)m->nrow));
    ELFEL_TRY(reduce_dense(c, tp, tstore.p, tvec.p));
    add_k<<<grid_for(m->nrow, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(m->rhs.p, tvec.p, m->nrow);
    ELFEL_LAUNCH_CHECK(c);
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    tp.release(c);
    edges.release(c);
    edofs.release(c);
    tstore.release(c);
    tvec.release(c);
  }
  return ELFEL_OK;
}

extern "C" int elfel_fused_stokes(elfel_sysmat* m, double mu) {
  CHECK_FREE(m);
  Ctx* c = &m->h->c;
  if (!m->fused || m->F.physics != ELFEL_STOKES)
    return fail(c, ELFEL_ERR_STATE, "stokes: fused_setup(ELFEL_STOKES) first");
  cudaSetDevice(c->device);
  Fused& F = m->F;
  {
    Phase ph(c, "integrate_stokes");
    ELFEL_TRY(launch_stokes(c, F.nel, F.conn_u.p, F.xy_u.p, mu, F.ncurved, F.tab, F.kstore.p, F.pmass_store.p));
  }
  {
    Phase ph(c, "reduce_K");
    ELFEL_TRY(reduce_values(c, m->P, F.kstore.p, m->vals.p));
  }
  ELFEL_CUDA(c, cudaMemsetAsync(m->rhs.p, 0, sizeof(double) * m->nrow, c->stream));
  ELFEL_TRY(reduce_dense(c, F.pmpat, F.pmass_store.p, F.pmass_diag.p));
  m->has_rhs = 1;
  m->finished = 1;
  m->values_version++;
  return ELFEL_OK;
}
