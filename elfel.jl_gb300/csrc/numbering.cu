// DOF numbering on the device: numberdofs! of one or several spaces from
// their essential-BC masks, and the FEIterator DOF table of a space from its
// connectivity.
//
// numberfreedofs!(f, firstnum) (src/FEFields.jl:137-154) gives the free DOFs
// firstnum, firstnum+1, ... in term-major, component-minor order;
// numberdatadofs!(f, firstnum) (:164-177) numbers the data DOFs the same way.
// numberdofs!(fesps) (src/FESpaces.jl:250-259) numbers the free DOFs of
// space 1, 2, ... (space i starts after the highest free number of space
// i-1, or at 1 when that space has none), then the data DOFs of space 1
// (after the highest free number of the last space), 2, ... (after the
// highest data number of the previous space, or at 1).  Each number is an
// exclusive scan of the free (or data) mask plus the space's first number.
// The element DOF table follows _storedofs! (src/FEIterators.jl:161-171):
// node-major, component-minor.
#include <algorithm>

#include "sysmat.cuh"

namespace elfel {

namespace {

__global__ void mask_flags_k(const uint8_t* __restrict__ mask, int64_t n, int want_data, int32_t* __restrict__ flags) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flags[i] = ((mask[i] != 0) == (want_data != 0)) ? 1 : 0;
}

// 0-based DOF numbers: (first + rank - 1) with the 1-based first numbers
__global__ void assign_numbers_k(const uint8_t* __restrict__ mask, int64_t n, const int64_t* __restrict__ foff,
                                 const int64_t* __restrict__ doff, int64_t ffirst, int64_t dfirst,
                                 int32_t* __restrict__ num0) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    num0[i] = (int32_t)(mask[i] ? dfirst + doff[i] - 1 : ffirst + foff[i] - 1);
}

__global__ void element_dofs_k(const int32_t* __restrict__ conn, int64_t nel, int nn, int ncomp,
                               const int32_t* __restrict__ num0, int32_t* __restrict__ dofs) {
  const int64_t total = nel * nn * ncomp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t en = i / ncomp;  // element * nn + local node
    const int j = (int)(i - en * ncomp);
    dofs[i] = num0[(int64_t)conn[en] * ncomp + j];
  }
}

__global__ void one_based_k(const int32_t* __restrict__ a, int64_t n, int64_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)a[i] + 1;
}

}  // namespace

int number_spaces(Ctx* c, int ns, const uint8_t* const* mask, const int64_t* n, int32_t* const* num0,
                  int64_t* nfree) {
  std::vector<int64_t> F(ns), D(ns);
  std::vector<DBuf<int64_t>> foff(ns), doff(ns);
  DBuf<int32_t> flags;
  int64_t nmax = 1;
  for (int s = 0; s < ns; ++s) nmax = std::max(nmax, n[s]);
  ELFEL_TRY(flags.alloc(c, (size_t)nmax));
  for (int s = 0; s < ns; ++s) {
    ELFEL_TRY(foff[s].alloc(c, (size_t)n[s] + 1));
    ELFEL_TRY(doff[s].alloc(c, (size_t)n[s] + 1));
    for (int want = 0; want < 2; ++want) {
      int64_t* off = want ? doff[s].p : foff[s].p;
      if (n[s]) {
        mask_flags_k<<<grid_for(n[s], 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(mask[s], n[s], want,
                                                                                           flags.p);
        ELFEL_LAUNCH_CHECK(c);
        ELFEL_TRY(scan_counts_i32(c, flags.p, n[s], off));
      } else {
        ELFEL_CUDA(c, cudaMemsetAsync(off, 0, sizeof(int64_t), c->stream));
      }
    }
    ELFEL_CUDA(c, cudaMemcpyAsync(&F[s], foff[s].p + n[s], sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaMemcpyAsync(&D[s], doff[s].p + n[s], sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  }
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  // first numbers as numberdofs! chains them (highest number of the previous
  // space + 1, the highest being 0 for a space without such DOFs)
  std::vector<int64_t> ff(ns), df(ns);
  int64_t high = 0;
  for (int s = 0; s < ns; ++s) {
    ff[s] = high + 1;
    high = F[s] > 0 ? ff[s] + F[s] - 1 : 0;
  }
  for (int s = 0; s < ns; ++s) {
    df[s] = high + 1;
    high = D[s] > 0 ? df[s] + D[s] - 1 : 0;
  }
  int64_t tot = 0;
  for (int s = 0; s < ns; ++s) {
    tot += F[s];
    if (n[s])
      assign_numbers_k<<<grid_for(n[s], 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(
          mask[s], n[s], foff[s].p, doff[s].p, ff[s], df[s], num0[s]);
    ELFEL_LAUNCH_CHECK(c);
  }
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int s = 0; s < ns; ++s) {
    foff[s].release(c);
    doff[s].release(c);
  }
  flags.release(c);
  if (nfree) *nfree = tot;
  return ELFEL_OK;
}

int element_dofs(Ctx* c, const int32_t* conn, int64_t nel, int nn, int ncomp, const int32_t* num0, int32_t* dofs) {
  const int64_t total = nel * nn * ncomp;
  if (total == 0) return ELFEL_OK;
  element_dofs_k<<<grid_for(total, 256, (int64_t)c->sm_count * 16), 256, 0, c->stream>>>(conn, nel, nn, ncomp, num0,
                                                                                        dofs);
  ELFEL_LAUNCH_CHECK(c);
  return ELFEL_OK;
}

int numbers_to_host(Ctx* c, const int32_t* num0, int64_t n, int64_t* host) {
  if (n == 0 || !host) return ELFEL_OK;
  DBuf<int64_t> t;
  ELFEL_TRY(t.alloc(c, (size_t)n));
  one_based_k<<<grid_for(n, 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(num0, n, t.p);
  ELFEL_LAUNCH_CHECK(c);
  ELFEL_CUDA(c, cudaMemcpyAsync(host, t.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, c->stream));
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  t.release(c);
  return ELFEL_OK;
}

}  // namespace elfel
