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

#define ELFEL_ABI_VERSION 2

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
 * caller owns; out[r] = +0 plus vals[s] over rows[s] == r+1 in increasing s, the
 * same bits as elfel_sysvec_assemble (a row of negative zeros gives +0).  A row
 * number outside 1..nrow (any entry at all when nrow is 0) returns
 * ELFEL_ERR_ARG and leaves out unchanged.
 * Scratch: one fixed device array inside the library (about 16 MB, kept by
 * every GPU that loads the library until the process exits), so
 *   - sizes are limited to ELFEL_NOALLOC_MAX_ROWS rows and
 *     ELFEL_NOALLOC_MAX_ENTRIES entries; larger calls return ELFEL_ERR_ARG;
 *   - the first call on a device looks up the array's device address (once,
 *     with that device current);
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

/* Cell shape of the primary space's elements. */
enum elfel_shape {
  ELFEL_SHAPE_TRIANGLE = 0, /* FEH1_T3 / FEH1_T6 by nodes_per_elem (src/FElements.jl:225-288) */
  ELFEL_SHAPE_Q4 = 1,       /* FEH1_Q4, 4-node quadrilateral (src/FElements.jl:290-320) */
  ELFEL_SHAPE_T4 = 2        /* FEH1_T4, 4-node tetrahedron, 3-D coordinates (src/FElements.jl:357-386) */
};

/* One finite element space, flattened from the Julia objects: the mesh
 * connectivity and geometry (MeshCore incidence relation and "geom"
 * attribute) and the FEIterator DOF table (eldofs, src/FEIterators.jl:119,
 * gathered by _storedofs!, src/FEIterators.jl:161-171). */
typedef struct {
  int32_t nodes_per_elem; /* 3 = FEH1_T3, 6 = FEH1_T6, 4 = FEH1_Q4 or FEH1_T4 */
  int32_t ncomp;          /* nfecopies of the FESpace (src/FESpaces.jl:25-40) */
  int64_t nel;
  int64_t nnodes;
  const int64_t* conn;   /* nel x nodes_per_elem, 1-based node numbers, element-major */
  const double* xy;      /* nnodes x sdim coordinates (sdim of elfel_fused_desc; 2 for every space but T4) */
  const int64_t* eldofs; /* nel x (nodes_per_elem*ncomp) 1-based DOFs, node-major/component-minor */
} elfel_space;

typedef struct {
  int32_t physics;           /* enum elfel_physics */
  int32_t npts;              /* quadrature points of the rule */
  const double* qp_coords;   /* npts x manifold-dimension parametric coordinates (src/RefShapes.jl:85-361) */
  const double* qp_weights;  /* npts weights */
  int64_t ndofs;             /* size of K (all spaces) */
  elfel_space u;             /* heat/elasticity space, or the Stokes velocity space */
  elfel_space p;             /* Stokes pressure space (nodes_per_elem = 3); else zeroed */
  int32_t shape;             /* enum elfel_shape of u; Q4 and T4 take ELFEL_HEAT only */
  int32_t sdim;              /* coordinates per node of u: 2, or 3 for T4 (0 means 2) */
} elfel_fused_desc;

/* Upload the mesh and DOF tables and build the CSC pattern and the
 * slot-to-nonzero map once (device key sort).  Later elfel_fused_* calls
 * reuse them.  Triplet order is that of the reference's assemble! calls. */
ELFEL_API int elfel_fused_setup(elfel_sysmat* m, const elfel_fused_desc* d);
/* numberdofs!(fesps) of src/FESpaces.jl:250-259 on the device for nspaces
 * spaces with one field each: space s has nterms[s] terms of ncomp[s]
 * components and the essential-BC mask isdatum[s] (nterms x ncomp bytes,
 * term-major, nonzero = data DOF, as setebc! leaves FEField.isdatum).  Free
 * DOFs are numbered space by space, term-major/component-minor, then the data
 * DOFs (src/FEFields.jl:137-177), with the reference's chaining of first
 * numbers.  dofnums[s] (nterms x ncomp, may be NULL) receives the 1-based
 * numbers, *nfree (may be NULL) the number of unknowns. */
ELFEL_API int elfel_number_dofs(elfel_ctx* ctx, int32_t nspaces, const int64_t* nterms, const int32_t* ncomp,
                                const uint8_t* const* isdatum, int64_t* const* dofnums, int64_t* nfree);
/* Fused set-up with the DOF numbering on the device: numberdofs! of the
 * space (heat, elasticity) or of [velocity, pressure] (Stokes) from their
 * essential-BC masks (src/FESpaces.jl:250-259 -> src/FEFields.jl:137-177:
 * free DOFs term-major/component-minor, space by space, then the data DOFs),
 * and the FEIterator DOF tables built from the connectivity
 * (src/FEIterators.jl:161-171), so that no DOF table crosses the host link.
 * The spaces' eldofs pointers are not read.  isdatum_u: u.nnodes x u.ncomp
 * bytes, nonzero where setebc! fixed the DOF (isdatum_p likewise for the
 * Stokes pressure; else NULL).  d->ndofs must be the spaces' DOF total.
 * dofnums_u / dofnums_p (may be NULL): the 1-based numbers, as the FEField
 * dofnums arrays; *nfree (may be NULL): the number of unknowns. */
ELFEL_API int elfel_fused_setup_numbered(elfel_sysmat* m, const elfel_fused_desc* d, const uint8_t* isdatum_u,
                                         const uint8_t* isdatum_p, int64_t* dofnums_u, int64_t* dofnums_p,
                                         int64_t* nfree);
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

/* ------------------------------------------------------------------ device block meshes
 * Mesh generation and DOF numbering on the device for the block meshes the
 * reference's tests build with MeshSteward (T3block / T6block, e.g.
 * test/test_heat.jl:28-33), with the whole boundary fixed: the scalar heat
 * FESpace after setebc! on the boundary nodes and numberdofs!
 * (src/FESpaces.jl:250-259, 287-291) -- free DOFs 1..nu, then data DOFs,
 * both in node order -- with no host tables.  Node numbering, element order
 * and coordinates are those of the host generators (nodes x-fastest; T6 on
 * the refined grid; coordinates as numpy.linspace). */
typedef struct {
  int32_t nodes_per_elem; /* 3 (T3block) or 6 (T6block) */
  int32_t orientation;    /* 0: cells cut on their (i,j)-(i+1,j+1) diagonal; 1: alternate diagonals */
  int32_t nx, ny;         /* cells */
  double lx, ly;          /* the rectangle [0,lx] x [0,ly] */
  int32_t npts;           /* quadrature rule of the heat integration, as elfel_fused_desc */
  int32_t reserved;
  const double* qp_coords;
  const double* qp_weights;
} elfel_block_desc;
/* Fused heat set-up from a device-generated block mesh; *ndofs and *nu (may
 * be NULL) receive the sizes. */
ELFEL_API int elfel_fused_setup_block(elfel_sysmat* m, const elfel_block_desc* d, int64_t* ndofs, int64_t* nu);
/* Dirichlet vector of a block system: T[1:ndofs] = 0 at free DOFs and
 * c[0] + c[1] x + c[2] y + c[3] x^2 + c[4] x y + c[5] y^2 at the data DOFs. */
ELFEL_API int elfel_block_dirichlet(elfel_sysmat* m, const double* coef6, double* T);
/* The tables of a fused system back on the host, 1-based as elfel_fused_desc
 * takes them: conn[nel x nn], xy[nnodes x 2], eldofs[nel x nedof] of the
 * primary space; a NULL pointer skips that table. */
ELFEL_API int elfel_fused_tables(elfel_sysmat* m, int64_t* conn, double* xy, int64_t* eldofs);
/* Sizes of a fused system: elements, nodes of the primary space, DOFs. */
ELFEL_API int elfel_fused_dims(elfel_sysmat* m, int64_t* nel, int64_t* nnodes, int64_t* ndofs);
/* The tile reduction plan of a fused system's K pattern (no counterpart in
 * the reference; built at a T6 heat pattern's second assembly): tiles, the
 * distinct tile programs they read, tiles summed from the contributor lists,
 * runs of consecutive tiles reading one program (one CTA each; 0 when the
 * reduction runs one CTA per tile). All zero when no plan is built. */
ELFEL_API int elfel_sysmat_tile_stats(elfel_sysmat* m, int64_t* ntiles, int64_t* nprograms, int64_t* nfallback,
                                      int64_t* nruns);

/* ------------------------------------------------------------------ error integrals
 * evaluate_pressure_error / evaluate_velocity_error of test/test_stokes.jl:438-496
 * on the device: err = sqrt(sum_e sum_q w_q det J |u_h(x_q) - u_exact(x_q)|^2)
 * over the elements of a fused system's space 0 (the primary space: 1 or 2
 * components) or space 1 (the Taylor-Hood pressure, on the vertex triangles).
 * U: the system vector (ndofs values, host).  poly: 15 coefficients per
 * component of u_exact = sum c_ab x^a y^b, a + b <= 4, in the order
 * (0,0),(1,0),(0,1),(2,0),(1,1),(0,2),(3,0),(2,1),(1,2),(0,3),(4,0),(3,1),(2,2),(1,3),(0,4).
 * The quadrature rule is given as in elfel_fused_desc. */
ELFEL_API int elfel_error_l2(elfel_sysmat* m, const double* U, int32_t space, const double* poly, int32_t npts,
                   const double* qp_coords, const double* qp_weights, double* err);

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

/* ------------------------------------------------------------------ batched solve
 * No counterpart in the reference (which solves one system at a time with
 * `\`, test/test_heat.jl:75): many assembled systems iterate together, each
 * launch covering the row tiles of every active system, as captured CUDA
 * graphs.  Each system's arithmetic is independent of the others in the
 * batch, so its result is bit-identical alone and in any mix.  A system held
 * by a slot (from add until its result is taken) refuses calls that change
 * it, and its destroy. */
typedef struct elfel_batch elfel_batch;
/* method: ELFEL_PCG64 or ELFEL_PCG32_IR; capacity: slots (systems at once). */
ELFEL_API int elfel_batch_create(elfel_ctx* ctx, int32_t method, int32_t capacity, elfel_batch** out);
ELFEL_API int elfel_batch_destroy(elfel_batch* b);
/* Admit system m with the arguments of elfel_solve (T: nrow values, host);
 * *slot receives its slot. */
ELFEL_API int elfel_batch_add(elfel_batch* b, elfel_sysmat* m, const double* F, const double* T, int64_t nu,
                    double rtol, int32_t maxit, int32_t* slot);
/* Run `graphs` graph launches (a fixed number of iterations each) over all
 * active systems; *active = systems still iterating afterwards. */
ELFEL_API int elfel_batch_step(elfel_batch* b, int32_t graphs, int32_t* active);
/* Slots whose solve has finished and whose result is not yet taken: up to
 * cap of them in slots[], their count in *n. */
ELFEL_API int elfel_batch_done(elfel_batch* b, int32_t* slots, int32_t cap, int32_t* n);
/* Result of a finished slot: T (nrow values, host) gets x in T[1:nu] and the
 * data values in the rest; stats as elfel_solve (seconds = from add to the
 * step that saw it finish).  Frees the slot. */
ELFEL_API int elfel_batch_result(elfel_batch* b, int32_t slot, double* T, elfel_solve_stats* stats);

/* ------------------------------------------------------------------ serving
 * No counterpart in the reference.  A server takes heat solve requests --
 * the problem of test/test_heat.jl:89-111 on a T3/T6 block mesh of a
 * rectangle, with conductivity kappa, source Q and a Dirichlet polynomial on
 * the whole boundary -- as they arrive, and each elfel_server_step:
 *   admits queued requests (first come, first served) while a batch slot is
 *   free and the device-memory budget allows, reusing a resident idle system
 *   of the same mesh (mesh, pattern and solver structures stay on the device)
 *   or generating one on the device, evicting idle systems (least recently
 *   used) for room; assembles all admitted requests in batched launches;
 *   adds them to the batched solver, where they iterate together with the
 *   requests already running; runs graphs_per_step graph launches; and
 *   completes the requests that finished.
 * Times are seconds on the server clock (elfel_server_clock).  With
 * batched = 0 the server solves one request at a time through elfel_solve
 * (the plain path), for comparison. */
typedef struct elfel_server elfel_server;
typedef struct {
  int32_t method;          /* ELFEL_PCG32_IR or ELFEL_PCG64 */
  int32_t batched;         /* 1: batched solver; 0: one request at a time via elfel_solve */
  int32_t max_active;      /* requests iterating at once (batch slots) */
  int32_t graphs_per_step; /* graph launches per step */
  double rtol;             /* relative residual of every solve */
  int32_t maxit;
  int32_t keep_idle;       /* keep finished systems resident for reuse by the same mesh */
  int64_t mem_budget;      /* device bytes resident systems may hold; 0: the context's budget only */
} elfel_server_config;
typedef struct {
  int32_t nodes_per_elem; /* 3 or 6 */
  int32_t orientation;    /* as elfel_block_desc */
  int32_t nx, ny;
  double lx, ly;
  double kappa, Q;
  double dirichlet[6];    /* T = c0 + c1 x + c2 y + c3 x^2 + c4 x y + c5 y^2 on the boundary */
  double t_arrival;       /* arrival time on the server clock; < 0: now */
  int32_t keep_solution;  /* keep T (ndofs values) for elfel_server_solution */
  int32_t reserved;
} elfel_heat_request;
typedef struct {
  int64_t id;
  int32_t status;         /* ELFEL_OK or the error of this request */
  int32_t iterations, refinements, converged;
  double relres;          /* FP64 ||b - K_ff x|| / ||b|| */
  double t_arrival, t_admit, t_done;
  int64_t ndofs, nu, nel;
} elfel_serve_result;
typedef struct {
  int64_t submitted, completed, rejected;
  int64_t systems_created, systems_reused, systems_evicted;
  int64_t resident_systems, resident_bytes;
  int64_t graph_launches, solver_kernel_launches, kernel_launches;
  double busy_seconds;    /* host time spent inside elfel_server_step */
  /* its parts: creating systems (mesh, pattern), batched assembly, joining
   * the solver (solver structures, values, lifted rhs), graph launches with
   * the state readback, completing requests */
  double create_seconds, assemble_seconds, join_seconds, iterate_seconds, harvest_seconds;
} elfel_server_stats;
ELFEL_API int elfel_server_create(elfel_ctx* ctx, const elfel_server_config* cfg, elfel_server** out);
ELFEL_API int elfel_server_destroy(elfel_server* s);
ELFEL_API int elfel_server_clock(elfel_server* s, double* t);
ELFEL_API int elfel_server_submit(elfel_server* s, const elfel_heat_request* r, int64_t* id);
/* One step of the loop; *active: requests iterating, *queued: waiting. */
ELFEL_API int elfel_server_step(elfel_server* s, int32_t* active, int32_t* queued);
/* Completed requests since the last poll (up to cap; *n = how many returned). */
ELFEL_API int elfel_server_poll(elfel_server* s, elfel_serve_result* out, int32_t cap, int32_t* n);
/* The kept solution of a completed request (n = its ndofs); frees it. */
ELFEL_API int elfel_server_solution(elfel_server* s, int64_t id, double* T, int64_t n);
ELFEL_API int elfel_server_stats_read(elfel_server* s, elfel_server_stats* out);

/* Autotuner records of the context (batched grids, batched assembly CTA
 * size): line index (0-based) as "key: candidate=ms ..." with the chosen one
 * starred, and its index in *choice.  ELFEL_ERR_ARG past the last line.  The
 * tuner is on unless the environment sets ELFEL_TUNE=0. */
ELFEL_API int elfel_ctx_tuning(const elfel_ctx* ctx, int index, char* line, int cap, int32_t* choice);

/* Diagnostics (no counterpart in the reference): the device's FMA throughput
 * in TFLOP/s for bits = 32 or 64, timed with CUDA events on a full wave of
 * independent FMA chains -- the figure behind the FP64-bound reading of the
 * assembly kernels. */
ELFEL_API int elfel_ctx_fma_rate(elfel_ctx* ctx, int32_t bits, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* ELFEL_GPU_H */
