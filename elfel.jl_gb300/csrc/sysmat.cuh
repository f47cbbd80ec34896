// Device-resident sparse system: CSC pattern, slot map, values, rhs, solver data.
#pragma once
#include "common.cuh"
#include "integrate.cuh"

namespace elfel {

// One local-matrix kind appended per element, in the order of the reference's
// assemble! calls.  rows come from table R (nel x nr), columns from C (nel x nc).
//   transposed = 0: assemble!(am, lma)            -> slots column-major (i fastest)
//   transposed = 1: assemble!(am, transpose(lma)) -> parent entries row-major,
//                   row/col swapped (src/Assemblers.jl:109-114)
// Storage: values live in a per-element record of `store_per_elem` doubles.
//   store_off: offset of this block's (parent's) values in the record
//   sym = 1:   the block is symmetric and only j >= i is stored (i,j)->(min,max)
struct SlotBlock {
  const int32_t* R = nullptr;  // nullptr: every row number is 0 (a vector as a 1 x n matrix)
  const int32_t* C = nullptr;
  int nr = 0, nc = 0;
  int transposed = 0;
  int sym = 0;
  int slot_off = 0;   // offset of this block among the element's slots
  int store_off = 0;  // offset of the values this block reads
};

constexpr int kMaxBlocks = 4;

// Division of n < 2^31 by an invariant d >= 1 as a multiply-high, an add and
// a shift (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1,
// n / d = (umulhi(n, m) + n) >> s (the sum stays below 2^32 for n < 2^31).
struct FastDiv {
  uint32_t m = 1;
  int s = 0;
  void init(uint32_t d) {
    s = 0;
    while ((1ull << s) < d) ++s;
    m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << s) - d)) / d + 1);
  }
  __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
    return (__umulhi(n, m) + n) >> s;
#else
    return (uint32_t)((((uint64_t)n * m) >> 32) + n) >> s;
#endif
  }
};

struct SlotGen {
  int64_t nel = 0;
  int slots_per_elem = 0;   // S
  int store_per_elem = 0;   // values stored per element
  int nblocks = 0;
  SlotBlock b[kMaxBlocks];
  // COO mode (nblocks == 0): one slot per triplet
  const int32_t* I = nullptr;
  const int32_t* J = nullptr;
  int64_t ncoo = 0;
  int64_t total() const { return nblocks ? nel * (int64_t)slots_per_elem : ncoo; }
  // divisions of slot_rc (prepare() sets them; build_pattern does)
  FastDiv spe_div, nr_div[kMaxBlocks], nc_div[kMaxBlocks];
  void prepare() {
    if (!nblocks) return;
    spe_div.init((uint32_t)slots_per_elem);
    for (int k = 0; k < nblocks; ++k) {
      nr_div[k].init((uint32_t)(b[k].nr > 0 ? b[k].nr : 1));
      nc_div[k].init((uint32_t)(b[k].nc > 0 ? b[k].nc : 1));
    }
  }
};

// Column-major index within a symmetric nr x nr block stored as its upper
// triangle (i <= j), packed column by column: j*(j+1)/2 + i.
__host__ __device__ __forceinline__ int sym_index(int i, int j) {
  if (i > j) { int t = i; i = j; j = t; }
  return j * (j + 1) / 2 + i;
}

// The storage index of slot s alone (no table reads).
__device__ __forceinline__ int64_t slot_store(const SlotGen& g, int64_t s) {
  if (g.nblocks == 0) return s;
  const uint32_t su = (uint32_t)s, spe = (uint32_t)g.slots_per_elem;
  const uint32_t eu = g.spe_div.div(su);
  const int l = (int)(su - eu * spe);
  int bi = 0;
#pragma unroll
  for (int k = 1; k < kMaxBlocks; ++k)
    if (k < g.nblocks && l >= g.b[k].slot_off) bi = k;
  const SlotBlock& B = g.b[bi];
  const int t = l - B.slot_off;
  int i, j;
  if (!B.transposed) {
    j = (int)g.nr_div[bi].div((uint32_t)t);
    i = t - j * B.nr;
  } else {
    i = (int)g.nc_div[bi].div((uint32_t)t);
    j = t - i * B.nc;
  }
  const int loc = B.sym ? sym_index(i, j) : (i + j * B.nr);
  return (int64_t)eu * g.store_per_elem + B.store_off + loc;
}

// Block mode: the slots of one element come in runs that share a column --
// the nr slots of a local column of a plain block, the nc slots of a parent
// row of a transposed one ("column groups", groups_per_elem() per element).
__host__ __device__ __forceinline__ int groups_per_elem(const SlotGen& g) {
  int n = 0;
  for (int k = 0; k < g.nblocks; ++k) n += g.b[k].transposed ? g.b[k].nr : g.b[k].nc;
  return n;
}

// Column group q: its column, first slot, length, and the element's row table
// (rows of the group's slots: rtab[k], k < len; nullptr: all rows 0).
__device__ __forceinline__ void group_info(const SlotGen& g, int G, int64_t q, int32_t& col, int64_t& s0, int& len,
                                           const int32_t*& rtab) {
  const int64_t e = q / G;
  int lg = (int)(q - e * G);
  int bi = 0;
#pragma unroll
  for (int k = 0; k < kMaxBlocks; ++k) {
    if (k >= g.nblocks) break;
    const int ng = g.b[k].transposed ? g.b[k].nr : g.b[k].nc;
    if (lg < ng) {
      bi = k;
      break;
    }
    lg -= ng;
  }
  const SlotBlock& B = g.b[bi];
  const int64_t base = e * (int64_t)g.slots_per_elem + B.slot_off;
  if (!B.transposed) {  // local column lg: slots lg*nr + i, rows R[e][i]
    col = B.C[e * B.nc + lg];
    s0 = base + (int64_t)lg * B.nr;
    len = B.nr;
    rtab = B.R ? B.R + e * B.nr : nullptr;
  } else {  // parent row lg: slots lg*nc + j, column R[e][lg], rows C[e][j]
    col = B.R ? B.R[e * B.nr + lg] : 0;
    s0 = base + (int64_t)lg * B.nc;
    len = B.nc;
    rtab = B.C + e * B.nc;
  }
}

__device__ __forceinline__ void slot_rc(const SlotGen& g, int64_t s, int32_t& r, int32_t& c, int64_t& store) {
  if (g.nblocks == 0) {
    r = g.I[s];
    c = g.J[s];
    store = s;
    return;
  }
  // slot numbers stay below 2^31 (build_pattern checks): multiply-shift
  // divisions prepared on the host
  const uint32_t su = (uint32_t)s, spe = (uint32_t)g.slots_per_elem;
  const uint32_t eu = g.spe_div.div(su);
  const int64_t e = (int64_t)eu;
  const int l = (int)(su - eu * spe);
  int bi = 0;
#pragma unroll
  for (int k = 1; k < kMaxBlocks; ++k)
    if (k < g.nblocks && l >= g.b[k].slot_off) bi = k;
  const SlotBlock& B = g.b[bi];
  const int t = l - B.slot_off;
  int i, j;  // parent (row, col) index within the local matrix
  if (!B.transposed) {
    j = (int)g.nr_div[bi].div((uint32_t)t);
    i = t - j * B.nr;
    r = B.R ? B.R[e * B.nr + i] : 0;
    c = B.C[e * B.nc + j];
  } else {
    i = (int)g.nc_div[bi].div((uint32_t)t);  // parent row
    j = t - i * B.nc;                         // parent col
    r = B.C[e * B.nc + j];
    c = B.R ? B.R[e * B.nr + i] : 0;
  }
  const int loc = B.sym ? sym_index(i, j) : (i + j * B.nr);
  store = e * (int64_t)g.store_per_elem + B.store_off + loc;
}

// Nonzeros per reduction window: a warp reduces one window in four rounds of
// 32 lanes, the window's nonzeros taken in order of their contributor count.
constexpr int kReduceWindow = 128;

// Tile reduction plan of a pattern (tiles.cu).
constexpr int kTileThreads = 256;
constexpr int kTileMaxNz = 512;        // nonzeros of a tile
constexpr int kTileMaxContrib = 1024;  // contributions of a tile
constexpr int kTileMaxCols = 256;      // columns of a tile
constexpr int kTileMaxClass = 15;      // contributions of one nonzero (more: the tile takes the slow path)
constexpr int kTileMaxEl = 320;        // distinct elements of a tile
constexpr int kTileMaxS = 128;         // stored values per element record
constexpr int kTileTableBytes = 40960; // shared memory for the tile's value table
constexpr int kTileFallback = 1, kTileSplit = 2, kTileEmpty = 4;

struct TileHdr {
  int64_t p0;       // first nonzero of the tile (CSC position)
  int64_t q0;       // first contribution (cptr[p0])
  int64_t boff;     // byte offset of the tile's program in the blob array
  int32_t col0, ncols;
  int32_t nz, nc;   // nonzeros, contributions
  int32_t nel;      // distinct elements
  int32_t maxcnt;   // largest contributor count
  int32_t emin;     // smallest element
  int32_t flags;    // kTileFallback: summed from the contributor lists; kTileEmpty: no nonzero
  int32_t prog;     // tile whose program this tile reads (its representative)
  int32_t pad;
};

struct TilePlan {
  int built = 0;
  int S = 0, V = 0, emax = 0;  // record entries, value-table entries per element, elements per tile
  int maxblob = 0;             // bytes of the largest program
  int maxnel = 0;              // elements of the largest tile
  int64_t ntiles = 0, nprograms = 0, nfallback = 0;
  // runs of consecutive tiles that read one program (or are all beyond the
  // limits), at most runlen tiles each: (first tile, tiles)
  int64_t nruns = 0;
  int runlen = 0;
  DBuf<int2> runs;
  DBuf<TileHdr> hdr;
  // the distinct programs, each 16-byte aligned: count-class starts (uint16),
  // element offsets from the tile's smallest element (int32, ascending),
  // first codes in count order (uint32: position << 16 | table index),
  // further codes (uint16 table indices, class by class, contribution-major)
  DBuf<uint8_t> blob;
  void release(Ctx* c);
};

// CSC pattern with the contributor lists of each nonzero.
struct Pattern {
  int64_t nrow = 0, ncol = 0, nnz = 0, nslots = 0;
  DBuf<int64_t> colptr;   // ncol+1
  DBuf<int32_t> rowval;   // nnz, 0-based
  DBuf<int32_t> cptr;     // nnz+1: contributors of nonzero k are contrib[cptr[k] .. cptr[k+1])
  DBuf<int32_t> contrib;  // nslots: storage index of each contribution, ascending slot order
  DBuf<uint8_t> perm;     // per window of kReduceWindow nonzeros: their order by contributor count
  int reductions = 0;     // value reductions run on this pattern (perm is built for the second)
  TilePlan tiles;         // built on request (build_tile_plan)
  void release(Ctx* c) {
    tiles.release(c);
    colptr.release(c);
    rowval.release(c);
    cptr.release(c);
    contrib.release(c);
    perm.release(c);
    reductions = 0;
    nrow = ncol = nnz = nslots = 0;
  }
};

// Build the CSC pattern of the slots of `g` (nrow x ncol matrix).
int build_pattern(Ctx* c, const SlotGen& g, int64_t nrow, int64_t ncol, Pattern* P);

// vals_out[k] = sum of store[contrib[t]] over t in [cptr[k], cptr[k+1]), in order.
int reduce_values(Ctx* c, Pattern& P, const double* store, double* vals_out);
// Dense vector of a 1 x n pattern (the rhs): out[c] = contributions of column c.
int reduce_dense(Ctx* c, const Pattern& P, const double* store, double* out);

// The tile plan of P for element records of S stored values; map[s] (NULL:
// identity) is the value-table index of stored entry s, V the table size.
int build_tile_plan(Ctx* c, Pattern& P, int S, int V, const uint8_t* map);
// vals = the K values of P from element records (src: nel x S doubles), or,
// with t6r_bases, from the 8 bases per element of the exact-rational T6
// heat record; the same bits as reduce_values.
int tile_reduce(Ctx* c, const Pattern& P, const double* src, int t6r_bases, double* vals);

// One reduction of a batched launch (device array ordered by blk0).
constexpr int kRedJobThreads = 256;
struct RedJob {
  int64_t blk0;            // first CTA of this job
  int64_t n;               // items: nnz, or columns of a dense rhs
  const int64_t* colptr;   // dense rhs: the 1 x n pattern's column pointers; else null
  const int32_t* cptr;
  const int32_t* contrib;
  const double* store;
  double* out;
};
int reduce_batch(Ctx* c, const RedJob* jobs_dev, int njobs, int64_t blocks);

// Convert 1-based int64 indices to 0-based int32 with a range check.
int to_index32(Ctx* c, const int64_t* src_host, int64_t n, int64_t limit, DBuf<int32_t>* dst,
               const char* what);
// The same on stream st from a device-readable host array (host_device_ptr)
// into dst (n entries); entries outside 1..limit become 0 and set *bad
// (device), which the caller reads after the stream's work.
int to_index32_direct(Ctx* c, cudaStream_t st, const int64_t* src, int64_t n, int64_t limit, int32_t* dst, int* bad);
// n doubles from a device-readable host array to dst on stream st (copy
// engine for pinned memory, a copy kernel for pageable memory).
int copy_host_f64(Ctx* c, cudaStream_t st, const double* src, int pinned, int64_t n, double* dst);

// Fused-mode device data.
struct Fused {
  int physics = 0;
  int npts = 0;
  int shape = ELFEL_SHAPE_TRIANGLE;  // enum elfel_shape of the primary space
  int sdim = 2;                      // coordinates per node of the primary space
  QPTab tab;                         // triangles
  ShapeTab stab;                     // Q4 / T4
  int nn_u = 0, ncomp_u = 0, nn_p = 0;
  int64_t nel = 0, nnodes_u = 0, nnodes_p = 0;
  DBuf<int32_t> conn_u, conn_p;      // nel x nn, 0-based node ids
  DBuf<double> xy_u;                 // nnodes x sdim
  DBuf<int32_t> dofs_u, dofs_p;      // nel x nedof, 0-based DOFs
  DBuf<int32_t> zero_rows;           // nel x nedof zeros (row table of the rhs "matrix")
  DBuf<double> coef;                 // per-element coefficients
  DBuf<double> kstore;               // element matrix records, nel x store_per_elem
  DBuf<double> fstore;               // element vector records, nel x nedof
  SlotGen kgen, fgen;
  Pattern fpat;                      // F pattern: 1 x ndofs matrix
  DBuf<double> pmass_store;          // Stokes: pressure mass diagonal per element (nel x 3)
  Pattern pmpat;
  DBuf<double> pmass_diag;           // ndofs (nonzero at pressure DOFs only)
  int is_block = 0;                  // tables generated on the device from `block`
  elfel_block_desc block;
  DBuf<uint8_t> straight;            // nel: 1 = straight-sided element (of the current coordinates)
  int64_t ncurved = -1;              // elements without the flag (-1: not computed)
  int f_direct_ok = 0;               // T6 heat: no DOF is a midside node of more than two elements
  int fpat_built = 0;                // fpat is built on first use (ensure_fpat)
  void release(Ctx* c) {
    is_block = 0;
    f_direct_ok = 0;
    fpat_built = 0;
    shape = ELFEL_SHAPE_TRIANGLE;
    sdim = 2;
    ncurved = -1;
    straight.release(c);
    conn_u.release(c); conn_p.release(c); xy_u.release(c); dofs_u.release(c); dofs_p.release(c);
    zero_rows.release(c); coef.release(c); kstore.release(c); fstore.release(c);
    fpat.release(c); pmass_store.release(c); pmpat.release(c); pmass_diag.release(c);
  }
};

struct SolverData;  // defined in solve.cu

}  // namespace elfel

struct elfel_sysmat {
  elfel_ctx* h = nullptr;
  int started = 0, finished = 0;
  int64_t nrow = 0, ncol = 0;
  void* coo_stage = nullptr;  // COO mode: device buffers of the appended triplets
  elfel::Pattern P;
  elfel::DBuf<double> vals;  // nnz CSC values
  elfel::DBuf<double> rhs;   // nrow (fused mode)
  int has_rhs = 0;
  int fused = 0;
  elfel::Fused F;
  elfel::SolverData* solver = nullptr;
  uint64_t values_version = 0;  // bumped whenever vals change
  int busy = 0;                 // held by a batch slot (its solver data is in use)
  // recorded on the context stream when P (its colptr and rowval) is complete
  cudaEvent_t ev_pattern = nullptr;
  int pattern_recorded = 0;
};

namespace elfel {

// Slot generators, patterns and value buffers of a fused system whose tables
// (F.conn_u, F.xy_u, F.dofs_u; F.physics, nn, ncomp, nel, tab set) are on the device.
int fused_build(elfel_sysmat* m, int64_t ndofs);
// Builds the right-hand side's pattern (F.fgen) if it is not built yet; only
// assemblies that reduce load records need it.
int ensure_fpat(elfel_sysmat* m);

// numberdofs! of ns spaces on the device (numbering.cu): mask[s] (n[s]
// entries, term-major / component-minor, nonzero = data DOF) -> num0[s], the
// 0-based DOF numbers; *nfree = the free DOFs of all spaces.
int number_spaces(Ctx* c, int ns, const uint8_t* const* mask, const int64_t* n, int32_t* const* num0,
                  int64_t* nfree);
// dofs (nel x nn*ncomp, node-major / component-minor) = num0 of each node of conn.
int element_dofs(Ctx* c, const int32_t* conn, int64_t nel, int nn, int ncomp, const int32_t* num0, int32_t* dofs);
// host[0..n) = num0 + 1 (int64).
int numbers_to_host(Ctx* c, const int32_t* num0, int64_t n, int64_t* host);

// Device tables of a block mesh of the rectangle [0,lx] x [0,ly]: nodes,
// connectivity and the DOFs of a scalar field fixed on the whole boundary
// (free DOFs numbered first, both in node order).  Sizes out: nel, nnodes, nu.
int block_tables(Ctx* c, const elfel_block_desc& d, Fused* F, int64_t* nu);
// T[dof] = Dirichlet polynomial at the data DOFs' nodes, 0 at free DOFs
// (device vector of ndofs values).
int block_dirichlet(Ctx* c, const elfel_block_desc& d, const double* coef6, const Fused& F, double* T);
// The primary space's tables back on the host, 1-based (NULL skips one).
int tables_to_host(Ctx* c, const Fused& F, int64_t* conn, double* xy, int64_t* eldofs);

}  // namespace elfel
