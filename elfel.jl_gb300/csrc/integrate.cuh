// Element-integration kernels and their quadrature tables.
#pragma once
#include "common.cuh"

namespace elfel {

constexpr int kIntThreads = 128;  // elements per CTA
constexpr int kMaxQP = 16;

// Quadrature-point tables of one element type, passed by value to kernels.
// Values and parametric gradients follow src/FElements.jl:239-288 and are
// evaluated at the rule's points as QPIterator's __bfundata does
// (src/QPIterators.jl:14-50).
struct QPTab {
  int npts;
  int nn;
  double w[kMaxQP];
  double N[kMaxQP][6];
  double G[kMaxQP][6][2];
  double Np[kMaxQP][3];  // T3 basis (Taylor-Hood pressure) at the same points
  // reference tensors for straight-sided elements (index i*6 + j)
  double S[2][2][36];  // sum_q w_q G_i,a G_j,b
  double T[2][18];     // sum_q w_q Np_j G_i,a      (index i*3 + j)
  double P[6];         // sum_q w_q N_i
  double Mp[3];        // sum_q w_q Np_j^2
};

struct Mat3 {
  double a[3][3];
};

int make_tables(int nn, int npts, const double* pc, const double* w, QPTab* t);

// straight: per-element straight-sided flags of the geometry (launch_straight;
// unused for T3, whose elements always are); ncurved: the number of elements
// without the flag (0 selects the straight-only T6 kernel).  fglob non-null:
// the load vector is added into fglob (zeroed, indexed by the nel x 6 table
// dofs) instead of being written to fstore; allowed only when
// heat_f_direct() holds and no DOF is a midside node of more than two
// elements.
int launch_heat(Ctx* c, int nn, int64_t nel, const int32_t* conn, const double* xy, const double* kappa, double Q,
                const uint8_t* straight, int64_t ncurved, const QPTab& tab, double* kstore, double* fstore,
                const int32_t* dofs = nullptr, double* fglob = nullptr);
// True when every element of a T6 mesh takes the exact-rule straight-sided
// form, whose K record is determined by 8 bases (t6r_bases).
bool heat_bases_ok(int nn, int64_t ncurved, const QPTab& tab);
// The T6 heat integration writing the 8 bases per element (bases: nel x 8)
// instead of the 21-entry K records; the load vector as in launch_heat.
int launch_heat_bases(Ctx* c, int64_t nel, const int32_t* conn, const double* xy, const double* kappa, double Q,
                      const QPTab& tab, double* bases, double* fstore, const int32_t* dofs = nullptr,
                      double* fglob = nullptr);
// True when the heat load vector of a T6 mesh takes the exact form (zero at
// the vertices, Q det / 6 at the midside nodes) in the straight-only kernel.
bool heat_f_direct(int nn, int64_t ncurved, const QPTab& tab);
// Per-element straight-sided flags (1: every midside node is the exact
// midpoint of its edge) of a mesh and the count of curved elements;
// recomputed whenever the coordinates change.  Synchronises the stream.
int launch_straight(Ctx* c, int nn, int64_t nel, const int32_t* conn, const double* xy, uint8_t* flag,
                    int64_t* ncurved);

// One mesh of a batched heat integration (device array, ordered by blk0).
struct HeatJob {
  int64_t blk0;  // first CTA of this mesh
  int64_t nel;
  const int32_t* conn;
  const double* xy;
  const double* kappa;
  const uint8_t* straight;
  double Q;
  double* kstore;
  double* fstore;
};
// All meshes of jobs_dev (same element type nn and tables) in one launch of
// `blocks` CTAs of nt threads (64, 128 or 256; one element per thread).
int launch_heat_batch(Ctx* c, int nn, int nt, const HeatJob* jobs_dev, int njobs, int64_t blocks, const QPTab& tab);
// Quadrilateral and tetrahedron heat (FEH1_Q4, FEH1_T4).  Basis values and
// parametric gradients at the rule's points (src/FElements.jl:290-320,
// 357-386); P[j] = sum_q w_q N_j(q), W = sum_q w_q.
struct ShapeTab {
  int shape;  // ELFEL_SHAPE_Q4 or ELFEL_SHAPE_T4
  int npts;
  double w[kMaxQP];
  double N[kMaxQP][4];
  double G[kMaxQP][4][2];  // Q4 only (T4 gradients are constant)
  double P[4];
  double W;
};
int make_shape_tables(int shape, int npts, const double* pc, const double* w, ShapeTab* t);
// Element records of the heat weak form on Q4 (xy: nnodes x 2) or T4 (xy:
// nnodes x 3) meshes: kstore nel x 10 (upper triangle, column-packed), fstore nel x 4.
int launch_heat_shape(Ctx* c, const ShapeTab& tab, int64_t nel, const int32_t* conn, const double* xy,
                      const double* kappa, double Q, double* kstore, double* fstore);

// ncurved: curved elements of the geometry (0: the straight-sided tensor form).
int launch_elasticity(Ctx* c, int nn, int64_t nel, const int32_t* conn, const double* xy, const Mat3& D,
                      const double* bforce, int64_t ncurved, const QPTab& tab, double* kstore, double* fstore);
int launch_traction(Ctx* c, int64_t ntrac, const int32_t* edges, const int32_t* conn, int nn, const double* xy,
                    double t0, double t1, double* out);
int launch_stokes(Ctx* c, int64_t nel, const int32_t* conn, const double* xy, double mu, int64_t ncurved,
                  const QPTab& tab, double* kstore, double* pmass);

}  // namespace elfel
