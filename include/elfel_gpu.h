/*
 * elfel_gpu.h -- C ABI of the GB300 (sm_103a) element-integration, sparse
 * assembly and sparse-solve library that backs Elfel.jl's assembly API.
 *
 * Every entry point returns an int status (ELFEL_OK = 0).  On failure the
 * context keeps a message, read with elfel_ctx_last_error().  No C++
 * exception crosses this boundary.  All host arrays are owned by the caller;
 * sizes are queried first and the caller allocates (size-query-then-fill).
 * Numbering follows the reference: DOF and node numbers passed in and out
 * are 1-based Int64, sparse matrices are CSC with 1-based Int64 colptr and
 * rowval (SparseMatrixCSC{Float64,Int64}).
 *
 * Reference interfaces replaced (Elfel.jl v0.4.0, file:line):
 *   SysmatAssemblerSparse        src/Assemblers.jl:19-24, 58-60
 *   start!(::SysmatAssemblerSparse)   src/Assemblers.jl:67-78
 *   assemble!(::SysmatAssemblerSparse, r, c, v)        :85-90
 *   assemble!(::SysmatAssemblerSparse, ::LocalMatrixAssembler)            :97-102
 *   assemble!(::SysmatAssemblerSparse, ::Transpose{LocalMatrixAssembler}) :109-114
 *   finish!(::SysmatAssemblerSparse) -> SparseArrays.sparse              :121-123
 *   SysvecAssembler start!/assemble!/finish!   src/Assemblers.jl:170-230
 *   the user integrate! loops (fused on the device):
 *     heat        test/test_heat.jl:35-71
 *     elasticity  test/test_elasticity.jl:140-180
 *     Stokes TH   test/test_stokes.jl:629-668
 *   solve!(T, K, F, nu)  test/test_heat.jl:73-76 (K[1:nu,1:nu] \ (F - K*T)[1:nu])
 */
#ifndef ELFEL_GPU_H
#define ELFEL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ELFEL_ABI_VERSION 1

#if defined(__GNUC__)
#define ELFEL_API __attribute__((visibility("default")))
#else
#define ELFEL_API
#endif

enum elfel_status {
  ELFEL_OK = 0,
  ELFEL_ERR_ARG = 1,           /* invalid argument (size, index out of range, NULL) */
  ELFEL_ERR_CUDA = 2,          /* a CUDA call failed */
  ELFEL_ERR_BUDGET = 3,        /* device memory budget of the context exceeded */
  ELFEL_ERR_NOT_CONVERGED = 4, /* iterative solve hit its iteration cap */
  ELFEL_ERR_STATE = 5,         /* call out of order (e.g. finish before start) */
  ELFEL_ERR_TIMEOUT = 6,       /* a bounded device-side wait expired */
  ELFEL_ERR_UNSUPPORTED = 7    /* element/physics combination not provided */
};

typedef struct elfel_ctx elfel_ctx;       /* one device, one stream, a memory budget */
typedef struct elfel_sysmat elfel_sysmat; /* a device-resident assembled system K (+ F) */

/* ------------------------------------------------------------------ context */
ELFEL_API int elfel_abi_version(void);
/* Create a context on CUDA device `device`.  mem_budget_bytes = 0: no cap. */
ELFEL_API int elfel_ctx_create(int device, int64_t mem_budget_bytes, elfel_ctx** out);
ELFEL_API int elfel_ctx_destroy(elfel_ctx* ctx);
ELFEL_API const char* elfel_ctx_last_error(const elfel_ctx* ctx);
/* Bytes of device memory held now and at peak by this context. */
ELFEL_API int elfel_ctx_memory(const elfel_ctx* ctx, int64_t* in_use, int64_t* peak);
/* Use a caller-owned cudaStream_t (NULL restores the context's own stream). */
ELFEL_API int elfel_ctx_set_stream(elfel_ctx* ctx, void* cuda_stream);
ELFEL_API void* elfel_ctx_stream(const elfel_ctx* ctx);
ELFEL_API int elfel_ctx_synchronize(elfel_ctx* ctx);
/* Phase timing (no reference counterpart; replaces the @time calls of
 * examples/heat/poisson/t3.jl:72,78-79): enable = 1 clears and starts
 * recording CUDA events around every kernel phase on the context's stream,
 * enable = 0 stops.  profile_read returns, for the index-th distinct phase
 * name, the summed device milliseconds and the number of launches;
 * ELFEL_ERR_ARG past the last phase. */
ELFEL_API int elfel_ctx_profile(elfel_ctx* ctx, int enable);
ELFEL_API int elfel_ctx_profile_read(elfel_ctx* ctx, int index, char* name, int name_cap, double* total_ms,
                                     int64_t* count);

/* ------------------------------------- SysmatAssemblerSparse (COO mode) */
/* SysmatAssemblerSparse(0.0): src/Assemblers.jl:58-60 */
ELFEL_API int elfel_sysmat_create(elfel_ctx* ctx, elfel_sysmat** out);
ELFEL_API int elfel_sysmat_destroy(elfel_sysmat* m);
/* start!(self, nrow, ncol): src/Assemblers.jl:67-78.  Drops earlier triplets. */
ELFEL_API int elfel_sysmat_start(elfel_sysmat* m, int64_t nrow, int64_t ncol);
/* assemble!: src/Assemblers.jl:85-114.  Appends n triplets with 1-based row
 * and column numbers, in the order given (the order duplicates are summed). */
ELFEL_API int elfel_sysmat_assemble_coo(elfel_sysmat* m, const int64_t* rows, const int64_t* cols,
                              const double* vals, int64_t n);
/* finish!: src/Assemblers.jl:121-123.  Builds the CSC on the device with the
 * semantics of SparseArrays.sparse(I,J,V,m,n): duplicates summed in append
 * order, explicit zeros kept, rows sorted within each column. */
ELFEL_API int elfel_sysmat_finish(elfel_sysmat* m, int64_t* nnz);
ELFEL_API int elfel_sysmat_dims(const elfel_sysmat* m, int64_t* nrow, int64_t* ncol, int64_t* nnz);
/* Copy the CSC out (1-based): colptr[ncol+1], rowval[nnz], nzval[nnz]. */
ELFEL_API int elfel_sysmat_csc(elfel_sysmat* m, int64_t* colptr, int64_t* rowval, double* nzval);
/* Copy the assembled right-hand side F (length nrow) out; fused mode only. */
ELFEL_API int elfel_sysmat_rhs(elfel_sysmat* m, double* F);

/* ------------------------------------------------ SysvecAssembler (COO) */
/* start!(av, nrow); assemble!(av, i, v) for each of n entries; finish!(av):
 * src/Assemblers.jl:194-230.  out[nrow] receives the dense vector; entries
 * with equal row are summed in the order given. rows are 1-based. */
ELFEL_API int elfel_sysvec_assemble(elfel_ctx* ctx, int64_t nrow, const int64_t* rows, const double* vals,
                          int64_t n, double* out);

/* Allocation-free vector assembly.  No counterpart in the reference: it is
 * elfel_sysvec_assemble for callers that cannot allocate device memory where
 * they assemble -- programs that give the library only memory their own
 * runtime manages, or loops that must not call cudaMalloc because it
 * synchronises the device and takes unbounded time.  rows (1-based) and vals
 * (n entries) are device pointers, out (nrow doubles) is a device pointer the
 * caller owns; out[r] = sum of vals[s] over rows[s] == r+1 in increasing s, the
 * same bits as elfel_sysvec_assemble.
 * Scratch: one fixed device array inside the library (about 16 MB, kept by
 * every GPU that loads the library until the process exits), so
 *   - sizes are limited to ELFEL_NOALLOC_MAX_ROWS rows and
 *     ELFEL_NOALLOC_MAX_ENTRIES entries; larger calls return ELFEL_ERR_ARG;
 *   - the first call on a device looks up the array's device address (once,
 *     with that device current); make that first call before any stream
 *     capture;
 *   - every call reuses the same array, which keeps the previous call's
 *     contents; calls whose work overlaps on the GPU (other streams, other
 *     contexts on the same device) race on it.
 * Work runs on the context's stream; the call synchronises that stream to
 * report out-of-range rows.  It calls no cudaMalloc, cudaFree or other
 * allocating routine. */
#define ELFEL_NOALLOC_MAX_ROWS 524288
#define ELFEL_NOALLOC_MAX_ENTRIES 2097152
ELFEL_API int elfel_sysvec_assemble_noalloc(elfel_ctx* ctx, int64_t nrow, const int64_t* rows, const double* vals,
                                            int64_t n, double* out);

/* ------------------------------------------------ fused (device) assembly */
enum elfel_physics {
  ELFEL_HEAT = 1,       /* test/test_heat.jl:41-58, per-element conductivity */
  ELFEL_ELASTICITY = 2, /* test/test_elasticity.jl:150-171, 2-component space */
  ELFEL_STOKES = 3      /* test/test_stokes.jl:629-657, vector T6 velocity + T3 pressure */
};

/* One finite element space on a triangle mesh, flattened from the Julia
 * objects: the mesh connectivity and geometry (MeshCore incidence relation and
 * "geom" attribute) and the FEIterator DOF table (eldofs, src/FEIterators.jl:119,
 * gathered by _storedofs!, src/FEIterators.jl:161-171). */
typedef struct {
  int32_t nodes_per_elem; /* 3 = FEH1_T3, 6 = FEH1_T6 (src/FElements.jl:225-288) */
  int32_t ncomp;          /* nfecopies of the FESpace (src/FESpaces.jl:25-40) */
  int64_t nel;
  int64_t nnodes;
  const int64_t* conn;   /* nel x nodes_per_elem, 1-based node numbers, element-major */
  const double* xy;      /* nnodes x 2 coordinates */
  const int64_t* eldofs; /* nel x (nodes_per_elem*ncomp) 1-based DOFs, node-major/component-minor */
} elfel_space;

typedef struct {
  int32_t physics;           /* enum elfel_physics */
  int32_t npts;              /* quadrature points of the triangle rule */
  const double* qp_coords;   /* npts x 2 parametric coordinates (src/RefShapes.jl:113-160) */
  const double* qp_weights;  /* npts weights */
  int64_t ndofs;             /* size of K (all spaces) */
  elfel_space u;             /* heat/elasticity space, or the Stokes velocity space */
  elfel_space p;             /* Stokes pressure space (nodes_per_elem = 3); else zeroed */
} elfel_fused_desc;

/* Upload the mesh and DOF tables and build the CSC pattern and the
 * slot-to-nonzero map once (device key sort).  Later elfel_fused_* calls
 * reuse them.  Triplet order is that of the reference's assemble! calls. */
ELFEL_API int elfel_fused_setup(elfel_sysmat* m, const elfel_fused_desc* d);
/* Replace the node coordinates of the primary space (same mesh topology). */
ELFEL_API int elfel_fused_set_geometry(elfel_sysmat* m, const double* xy);
/* Heat: K and F for conductivity kappa[nel] (NULL: keep the resident values
 * from the previous call) and heat source Q. */
ELFEL_API int elfel_fused_heat(elfel_sysmat* m, const double* kappa, double Q);
/* Elasticity with isotropic material (E, nu), plane_strain = 1 for plane
 * strain, 0 for plane stress; body force per element bforce[nel x 2] (NULL =
 * none); traction on boundary edges: trac_edges[ntrac x nedge_nodes] 1-based
 * node numbers (2 for T3, 3 for T6 with the midside node last), traction[2]. */
ELFEL_API int elfel_fused_elasticity(elfel_sysmat* m, double E, double nu, int32_t plane_strain,
                           const double* bforce, const int64_t* trac_edges, int64_t ntrac,
                           const double* traction);
/* Stokes (vector Laplacian Taylor-Hood): K with the uu, up and up' blocks,
 * F = 0, plus the pressure mass-matrix diagonal kept for preconditioning. */
ELFEL_API int elfel_fused_stokes(elfel_sysmat* m, double mu);

/* ------------------------------------------------------------------ solve */
enum elfel_solver {
  ELFEL_PCG64 = 0,      /* Jacobi-PCG, all FP64 */
  ELFEL_PCG32_IR = 1,   /* FP32 Jacobi-CG with FP64 residual replacement (iterative refinement) */
  ELFEL_MINRES64 = 2,   /* block-diagonal preconditioned MINRES, FP64 (saddle-point systems) */
  ELFEL_MINRES32_IR = 3 /* FP32 MINRES inside FP64 iterative refinement */
};

typedef struct {
  int32_t iterations;  /* inner iterations in total */
  int32_t refinements; /* FP64 residual replacements / outer steps */
  int32_t converged;   /* 1 if the relative residual reached rtol */
  int32_t reserved;
  double relres;       /* final ||b - A x|| / ||b|| computed in FP64 */
  double seconds;      /* device time of the solve */
} elfel_solve_stats;

/* solve!(T, K, F, nu) of test/test_heat.jl:73-76:
 *   T[1:nu] = K[1:nu,1:nu] \ (F[1:nu] - (K*T)[1:nu])
 * T (length nrow) is read (data values) and overwritten in its first nu
 * entries.  F = NULL uses the device right-hand side of the fused assembly. */
ELFEL_API int elfel_solve(elfel_sysmat* m, const double* F, double* T, int64_t nu, int32_t method,
                double rtol, int32_t maxit, elfel_solve_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* ELFEL_GPU_H */
