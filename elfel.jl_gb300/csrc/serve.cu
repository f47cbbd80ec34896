// Serving loop for heat solve requests on block meshes.  No counterpart in
// the reference (a script assembles and solves one problem at a time,
// Elfel.jl test/test_heat.jl:89-111); each request here is that script's
// problem: a T3/T6 block mesh of a rectangle, conductivity kappa, source Q
// and a Dirichlet polynomial on the whole boundary.
//
// A step of the loop:
//   1. admission: queued requests, first come first served, while a batch
//      slot is free and the device-memory budget allows.  A finished system
//      with the same mesh (element type, grid, rectangle, quadrature) is
//      reused -- mesh, pattern, slot map and SELL structure stay resident --
//      else a new one is generated on the device, evicting idle systems
//      (least recently used) when the budget needs room;
//   2. batched assembly of everything admitted in this step: one launch per
//      element type integrates all their elements, one launch reduces all
//      their K values and rhs entries (flattened job tables);
//   3. the admitted systems join the batched solver (continuous batching:
//      they iterate in the same graph launches as the requests already
//      running);
//   4. graph launches of the batched iterations;
//   5. harvest: finished requests get their FP64 residual, timestamps and,
//      when asked, their solution on the host; their systems go idle.
// With `batched` = 0 the server instead solves one request at a time through
// the one-system solver (the plain path a user calls), the reference point
// of the batched form.
#include <math.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <vector>

#include "integrate.cuh"
#include "solve.cuh"

namespace elfel {
int batch_add_dev(elfel_batch* b, elfel_sysmat* m, const double* F, const double* T, int t_dev, int64_t nu,
                  double rtol, int32_t maxit, int32_t* slot_out);
int batch_step(elfel_batch* b, int32_t graphs, int32_t* active);
int batch_take(elfel_batch* b, int32_t k, double* T_out, int t_dev, elfel_solve_stats* stats);
int batch_counts(elfel_batch* b, int64_t* launches, int64_t* kernels);
}  // namespace elfel

using namespace elfel;

namespace {

using Clock = std::chrono::steady_clock;

struct Key {
  int nn, orient, nx, ny;
  double lx, ly;
  bool operator<(const Key& o) const {
    if (nn != o.nn) return nn < o.nn;
    if (orient != o.orient) return orient < o.orient;
    if (nx != o.nx) return nx < o.nx;
    if (ny != o.ny) return ny < o.ny;
    if (lx != o.lx) return lx < o.lx;
    return ly < o.ly;
  }
};

struct Req {
  int64_t id;
  elfel_heat_request r;
  double t_arrival;
};

// A resident system: one block mesh with its pattern, solver structures and
// the Dirichlet vector of its current request.
struct Sys {
  Key key;
  elfel_sysmat* m = nullptr;
  int64_t bytes = 0;
  int64_t nel = 0, n = 0, nu = 0;
  DBuf<double> T;  // Dirichlet values (device)
  bool busy = false;
  Clock::time_point last_used;
  Req req;
  double t_admit = 0.0;
  int32_t slot = -1;
};

// 3-point triangle rule (exact for quadratics) and the 1-point rule, as
// quadrature(RefShapeTriangle, (npts = ...)) of src/RefShapes.jl:113-119
const double kQP3[6] = {2.0 / 3, 1.0 / 6, 1.0 / 6, 2.0 / 3, 1.0 / 6, 1.0 / 6};
const double kW3[3] = {1.0 / 3 / 2, 1.0 / 3 / 2, 1.0 / 3 / 2};
const double kQP1[2] = {1.0 / 3.0, 1.0 / 3.0};
const double kW1[1] = {1.0 / 2.0};

__global__ void fill_k(double* a, int64_t n, double v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = v;
}

}  // namespace

struct elfel_server {
  elfel_ctx* h = nullptr;
  elfel_server_config cfg;
  elfel_batch* batch = nullptr;
  Clock::time_point t0;
  int64_t next_id = 1;
  std::deque<Req> pending;
  std::list<std::unique_ptr<Sys>> systems;  // resident (busy or idle)
  std::map<int32_t, Sys*> by_slot;
  std::vector<elfel_serve_result> finished;
  std::map<int64_t, std::vector<double>> solutions;
  std::map<Key, int64_t> key_bytes;  // measured size of a system per mesh
  double bytes_per_elem[7] = {0, 0, 0, 1200.0, 0, 0, 2600.0};  // first guesses, then measured
  int64_t held = 0;                  // bytes of resident systems
  elfel_server_stats st;
  DBuf<HeatJob> hjobs;
  DBuf<RedJob> rjobs;
};

namespace {

double now_s(const elfel_server* s) { return std::chrono::duration<double>(Clock::now() - s->t0).count(); }

// Adds the host time of a scope to a counter.
struct Timed {
  double& acc;
  Clock::time_point a = Clock::now();
  explicit Timed(double& t) : acc(t) {}
  ~Timed() { acc += std::chrono::duration<double>(Clock::now() - a).count(); }
};

Key key_of(const elfel_heat_request& r) { return Key{r.nodes_per_elem, r.orientation, r.nx, r.ny, r.lx, r.ly}; }

int64_t estimate(elfel_server* s, const Key& k) {
  auto it = s->key_bytes.find(k);
  if (it != s->key_bytes.end()) return it->second;
  return (int64_t)(s->bytes_per_elem[k.nn] * 2.0 * k.nx * k.ny) + (1 << 20);
}

void destroy_sys(elfel_server* s, Sys* y) {
  Ctx* c = &s->h->c;
  y->T.release(c);
  if (y->m) elfel_sysmat_destroy(y->m);
  y->m = nullptr;
  s->held -= y->bytes;
  s->st.resident_bytes = s->held;
}

// Drop the least recently used idle system; false when none is idle.
bool evict_one(elfel_server* s) {
  auto victim = s->systems.end();
  for (auto it = s->systems.begin(); it != s->systems.end(); ++it)
    if (!(*it)->busy && (victim == s->systems.end() || (*it)->last_used < (*victim)->last_used)) victim = it;
  if (victim == s->systems.end()) return false;
  destroy_sys(s, victim->get());
  s->systems.erase(victim);
  s->st.systems_evicted++;
  s->st.resident_systems = (int64_t)s->systems.size();
  return true;
}

Sys* take_idle(elfel_server* s, const Key& k) {
  Sys* best = nullptr;
  for (auto& y : s->systems)
    if (!y->busy && !(y->key < k) && !(k < y->key)) {
      best = y.get();
      break;
    }
  return best;
}

int create_sys(elfel_server* s, const Key& k, int npts, Sys** out) {
  Ctx* c = &s->h->c;
  Timed tm(s->st.create_seconds);
  const int64_t before = c->in_use;
  std::unique_ptr<Sys> y(new Sys());
  y->key = k;
  ELFEL_TRY(elfel_sysmat_create(s->h, &y->m));
  elfel_block_desc d;
  memset(&d, 0, sizeof(d));
  d.nodes_per_elem = k.nn;
  d.orientation = k.orient;
  d.nx = k.nx;
  d.ny = k.ny;
  d.lx = k.lx;
  d.ly = k.ly;
  d.npts = npts;
  d.qp_coords = npts == 1 ? kQP1 : kQP3;
  d.qp_weights = npts == 1 ? kW1 : kW3;
  int64_t n = 0, nu = 0;
  int rc = elfel_fused_setup_block(y->m, &d, &n, &nu);
  if (rc == ELFEL_OK) rc = y->T.alloc(c, (size_t)std::max<int64_t>(n, 1));
  if (rc != ELFEL_OK) {
    y->T.release(c);
    elfel_sysmat_destroy(y->m);
    return rc;
  }
  y->n = n;
  y->nu = nu;
  y->nel = y->m->F.nel;
  y->bytes = c->in_use - before;  // grows again when the solver data is built
  s->held += y->bytes;
  s->st.systems_created++;
  *out = y.get();
  s->systems.push_back(std::move(y));
  s->st.resident_systems = (int64_t)s->systems.size();
  s->st.resident_bytes = s->held;
  return ELFEL_OK;
}

// Integrate the heat elements of all systems in ys with one launch per element
// type; the autotuner picks the CTA size per type and size bucket.
int assemble_batch(elfel_server* s, const std::vector<Sys*>& ys) {
  Ctx* c = &s->h->c;
  if (ys.empty()) return ELFEL_OK;
  Timed tm(s->st.assemble_seconds);
  for (Sys* y : ys) {
    Fused& F = y->m->F;
    fill_k<<<grid_for(F.nel, 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(F.coef.p, F.nel, y->req.r.kappa);
    ELFEL_LAUNCH_CHECK(c);
  }
  s->st.kernel_launches += (int64_t)ys.size();
  for (int nn : {3, 6}) {
    for (int npts : {1, 3}) {
      std::vector<Sys*> grp;
      int64_t nel = 0;
      for (Sys* y : ys)
        if (y->key.nn == nn && y->m->F.npts == npts) {
          grp.push_back(y);
          nel += y->nel;
        }
      if (grp.empty()) continue;
      const QPTab& tab = grp[0]->m->F.tab;
      int bucket = 0;
      while ((1LL << (bucket + 1)) <= nel) ++bucket;
      char key[64];
      snprintf(key, sizeof(key), "heat_batch_T%d_q%d_elems_2^%d", nn, npts, bucket);
      const int cand[3] = {128, 64, 256};
      int choice = tune_lookup(c, key);
      auto launch = [&](int nt) -> int {
        std::vector<HeatJob> jobs;
        int64_t blk = 0;
        for (Sys* y : grp) {
          Fused& F = y->m->F;
          HeatJob j;
          j.blk0 = blk;
          j.nel = F.nel;
          j.conn = F.conn_u.p;
          j.xy = F.xy_u.p;
          j.kappa = F.coef.p;
          j.straight = F.straight.p;
          j.Q = y->req.r.Q;
          j.kstore = F.kstore.p;
          j.fstore = F.fstore.p;
          jobs.push_back(j);
          blk += (F.nel + nt - 1) / nt;
        }
        ELFEL_TRY(s->hjobs.ensure(c, jobs.size()));
        ELFEL_CUDA(c, cudaMemcpyAsync(s->hjobs.p, jobs.data(), sizeof(HeatJob) * jobs.size(), cudaMemcpyHostToDevice,
                                      c->stream));
        ELFEL_TRY(launch_heat_batch(c, nn, nt, s->hjobs.p, (int)jobs.size(), blk, tab));
        s->st.kernel_launches++;
        // the job table must stay alive until the launch has read it
        ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
        return ELFEL_OK;
      };
      if (choice < 0 && c->tune && nel >= 65536) {
        std::vector<double> ms(3, 0.0);
        cudaEvent_t e0, e1;
        ELFEL_CUDA(c, cudaEventCreate(&e0));
        ELFEL_CUDA(c, cudaEventCreate(&e1));
        for (int k = 0; k < 3; ++k) {
          ELFEL_CUDA(c, cudaEventRecord(e0, c->stream));
          ELFEL_TRY(launch(cand[k]));
          ELFEL_CUDA(c, cudaEventRecord(e1, c->stream));
          ELFEL_CUDA(c, cudaEventSynchronize(e1));
          float t = 0.f;
          cudaEventElapsedTime(&t, e0, e1);
          ms[k] = t;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        choice = (int)(std::min_element(ms.begin(), ms.end()) - ms.begin());
        tune_record(c, key, "128,64,256", choice, ms);
      }
      ELFEL_TRY(launch(cand[choice < 0 ? 0 : choice]));
    }
  }
  // K values and rhs of all systems in one launch
  for (Sys* y : ys) ELFEL_TRY(ensure_fpat(y->m));
  std::vector<RedJob> rj;
  int64_t blk = 0;
  for (Sys* y : ys) {
    elfel_sysmat* m = y->m;
    RedJob a;
    a.blk0 = blk;
    a.n = m->P.nnz;
    a.colptr = nullptr;
    a.cptr = m->P.cptr.p;
    a.contrib = m->P.contrib.p;
    a.store = m->F.kstore.p;
    a.out = m->vals.p;
    if (a.n > 0) {
      rj.push_back(a);
      blk += (a.n + kRedJobThreads - 1) / kRedJobThreads;
    }
    RedJob f;
    f.blk0 = blk;
    f.n = m->F.fpat.ncol;
    f.colptr = m->F.fpat.colptr.p;
    f.cptr = m->F.fpat.cptr.p;
    f.contrib = m->F.fpat.contrib.p;
    f.store = m->F.fstore.p;
    f.out = m->rhs.p;
    if (f.n > 0) {
      rj.push_back(f);
      blk += (f.n + kRedJobThreads - 1) / kRedJobThreads;
    }
  }
  ELFEL_TRY(s->rjobs.ensure(c, std::max<size_t>(rj.size(), 1)));
  ELFEL_CUDA(c, cudaMemcpyAsync(s->rjobs.p, rj.data(), sizeof(RedJob) * rj.size(), cudaMemcpyHostToDevice, c->stream));
  ELFEL_TRY(reduce_batch(c, s->rjobs.p, (int)rj.size(), blk));
  s->st.kernel_launches++;
  for (Sys* y : ys) {
    ELFEL_TRY(block_dirichlet(c, y->m->F.block, y->req.r.dirichlet, y->m->F, y->T.p));
    elfel_sysmat* m = y->m;
    m->has_rhs = 1;
    m->finished = 1;
    m->values_version++;
  }
  s->st.kernel_launches += (int64_t)ys.size();
  ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
  return ELFEL_OK;
}

void reject(elfel_server* s, const Req& q, int code) {
  elfel_serve_result r;
  memset(&r, 0, sizeof(r));
  r.id = q.id;
  r.status = code;
  r.t_arrival = q.t_arrival;
  r.t_admit = r.t_done = now_s(s);
  s->finished.push_back(r);
  s->st.rejected++;
}

void release_sys(elfel_server* s, Sys* y) {
  y->busy = false;
  y->slot = -1;
  y->last_used = Clock::now();
  if (!s->cfg.keep_idle) {
    for (auto it = s->systems.begin(); it != s->systems.end(); ++it)
      if (it->get() == y) {
        destroy_sys(s, y);
        s->systems.erase(it);
        break;
      }
    s->st.resident_systems = (int64_t)s->systems.size();
  }
}

int finish_request(elfel_server* s, Sys* y, const elfel_solve_stats& sst, int status, std::vector<double>* sol) {
  elfel_serve_result r;
  memset(&r, 0, sizeof(r));
  r.id = y->req.id;
  r.status = status;
  r.iterations = sst.iterations;
  r.refinements = sst.refinements;
  r.converged = sst.converged;
  r.relres = sst.relres;
  r.t_arrival = y->req.t_arrival;
  r.t_admit = y->t_admit;
  r.t_done = now_s(s);
  r.ndofs = y->n;
  r.nu = y->nu;
  r.nel = y->nel;
  s->finished.push_back(r);
  s->st.completed++;
  if (sol && y->req.r.keep_solution) s->solutions[r.id] = std::move(*sol);
  release_sys(s, y);
  return ELFEL_OK;
}

int admit(elfel_server* s, std::vector<Sys*>* admitted) {
  int active = (int)s->by_slot.size();
  while (!s->pending.empty() && active + (int)admitted->size() < s->cfg.max_active) {
    const Req q = s->pending.front();
    const Key k = key_of(q.r);
    Sys* y = take_idle(s, k);
    if (y) {
      s->st.systems_reused++;
    } else {
      const int64_t est = estimate(s, k);
      if (s->cfg.mem_budget > 0) {
        while (s->held + est > s->cfg.mem_budget && evict_one(s)) {
        }
        if (s->held + est > s->cfg.mem_budget) {
          if (active > 0 || !admitted->empty()) break;  // wait until running requests free memory
          if (est > s->cfg.mem_budget) {  // can never fit
            s->pending.pop_front();
            reject(s, q, ELFEL_ERR_BUDGET);
            continue;
          }
        }
      }
      int rc = create_sys(s, k, 3, &y);
      if (rc == ELFEL_ERR_BUDGET) {  // the context's own cap: free idle systems and retry
        while (rc == ELFEL_ERR_BUDGET && evict_one(s)) rc = create_sys(s, k, 3, &y);
      }
      if (rc == ELFEL_ERR_BUDGET && (active > 0 || !admitted->empty())) break;
      if (rc != ELFEL_OK) {
        s->pending.pop_front();
        reject(s, q, rc);
        continue;
      }
    }
    s->pending.pop_front();
    y->busy = true;
    y->req = q;
    y->t_admit = now_s(s);
    admitted->push_back(y);
  }
  return ELFEL_OK;
}

int step_batched(elfel_server* s, int32_t* active) {
  Ctx* c = &s->h->c;
  std::vector<Sys*> adm;
  ELFEL_TRY(admit(s, &adm));
  ELFEL_TRY(assemble_batch(s, adm));
  for (Sys* y : adm) {
    Timed tm(s->st.join_seconds);
    const int64_t before = c->in_use;
    int32_t slot = -1;
    int rc = batch_add_dev(s->batch, y->m, nullptr, y->T.p, 1, y->nu, s->cfg.rtol, s->cfg.maxit, &slot);
    if (rc != ELFEL_OK) {
      elfel_solve_stats z;
      memset(&z, 0, sizeof(z));
      finish_request(s, y, z, rc, nullptr);
      continue;
    }
    // the first solve of a system builds its solver data: count it as resident
    const int64_t grown = c->in_use - before;
    y->bytes += grown;
    s->held += grown;
    s->key_bytes[y->key] = y->bytes;
    const double per = (double)y->bytes / (double)std::max<int64_t>(y->nel, 1);
    if (per > s->bytes_per_elem[y->key.nn] || s->key_bytes.size() == 1) s->bytes_per_elem[y->key.nn] = per;
    s->st.resident_bytes = s->held;
    y->slot = slot;
    s->by_slot[slot] = y;
  }
  int32_t act = 0;
  if (!s->by_slot.empty()) {
    Timed tm(s->st.iterate_seconds);
    ELFEL_TRY(batch_step(s->batch, s->cfg.graphs_per_step, &act));
  }
  // harvest
  Timed tm(s->st.harvest_seconds);
  int32_t nd = 0;
  std::vector<int32_t> ready(s->cfg.max_active);
  ELFEL_TRY(elfel_batch_done(s->batch, ready.data(), (int32_t)ready.size(), &nd));
  for (int i = 0; i < std::min<int>(nd, (int)ready.size()); ++i) {
    const int32_t slot = ready[i];
    auto it = s->by_slot.find(slot);
    if (it == s->by_slot.end()) continue;
    Sys* y = it->second;
    std::vector<double> sol;
    double* dst = nullptr;
    if (y->req.r.keep_solution) {
      sol.resize((size_t)y->n);
      dst = sol.data();
    }
    elfel_solve_stats sst;
    const int rc = batch_take(s->batch, slot, dst, 0, &sst);
    s->by_slot.erase(it);
    ELFEL_TRY(finish_request(s, y, sst, rc, &sol));
  }
  if (active) *active = (int32_t)s->by_slot.size();
  return ELFEL_OK;
}

// One request at a time through the one-system solver.
int step_plain(elfel_server* s, int32_t* active) {
  Ctx* c = &s->h->c;
  std::vector<Sys*> adm;
  const int cap = s->cfg.max_active;
  s->cfg.max_active = 1;
  int rc = admit(s, &adm);
  s->cfg.max_active = cap;
  ELFEL_TRY(rc);
  ELFEL_TRY(assemble_batch(s, adm));
  for (Sys* y : adm) {
    Timed tm(s->st.iterate_seconds);
    const int64_t before = c->in_use;
    std::vector<double> T((size_t)y->n);
    ELFEL_CUDA(c, cudaMemcpyAsync(T.data(), y->T.p, sizeof(double) * y->n, cudaMemcpyDeviceToHost, c->stream));
    ELFEL_CUDA(c, cudaStreamSynchronize(c->stream));
    elfel_solve_stats sst;
    memset(&sst, 0, sizeof(sst));
    const int src = elfel_solve(y->m, nullptr, T.data(), y->nu, s->cfg.method, s->cfg.rtol, s->cfg.maxit, &sst);
    const int64_t grown = c->in_use - before;
    y->bytes += grown;
    s->held += grown;
    s->key_bytes[y->key] = y->bytes;
    s->st.resident_bytes = s->held;
    ELFEL_TRY(finish_request(s, y, sst, src, &T));
  }
  if (active) *active = 0;
  return ELFEL_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" int elfel_server_create(elfel_ctx* h, const elfel_server_config* cfg, elfel_server** out) {
  if (!h || !cfg || !out) return ELFEL_ERR_ARG;
  Ctx* c = &h->c;
  if (cfg->method != ELFEL_PCG64 && cfg->method != ELFEL_PCG32_IR)
    return fail(c, ELFEL_ERR_UNSUPPORTED, "server: methods ELFEL_PCG64 and ELFEL_PCG32_IR");
  if (cfg->max_active < 1 || cfg->graphs_per_step < 1 || !(cfg->rtol > 0.0) || cfg->maxit < 1 || cfg->mem_budget < 0)
    return fail(c, ELFEL_ERR_ARG, "server: max_active, graphs_per_step, maxit >= 1, rtol > 0, mem_budget >= 0");
  elfel_server* s = new elfel_server();
  s->h = h;
  s->cfg = *cfg;
  s->t0 = Clock::now();
  memset(&s->st, 0, sizeof(s->st));
  if (cfg->batched) {
    const int rc = elfel_batch_create(h, cfg->method, cfg->max_active, &s->batch);
    if (rc != ELFEL_OK) {
      delete s;
      return rc;
    }
  }
  *out = s;
  return ELFEL_OK;
}

extern "C" int elfel_server_destroy(elfel_server* s) {
  if (!s) return ELFEL_OK;
  if (s->batch) elfel_batch_destroy(s->batch);
  Ctx* c = &s->h->c;
  for (auto& y : s->systems) {
    if (y->m) y->m->busy = 0;
    destroy_sys(s, y.get());
  }
  s->hjobs.release(c);
  s->rjobs.release(c);
  delete s;
  return ELFEL_OK;
}

extern "C" int elfel_server_clock(elfel_server* s, double* t) {
  if (!s || !t) return ELFEL_ERR_ARG;
  *t = now_s(s);
  return ELFEL_OK;
}

extern "C" int elfel_server_submit(elfel_server* s, const elfel_heat_request* r, int64_t* id) {
  if (!s || !r) return ELFEL_ERR_ARG;
  Ctx* c = &s->h->c;
  if ((r->nodes_per_elem != 3 && r->nodes_per_elem != 6) || (r->orientation != 0 && r->orientation != 1) ||
      r->nx < 1 || r->ny < 1 || !(r->lx > 0.0) || !(r->ly > 0.0) || !(r->kappa > 0.0))
    return fail(c, ELFEL_ERR_ARG, "submit: T3/T6, orientation 0/1, nx, ny >= 1, positive sizes and kappa");
  Req q;
  q.id = s->next_id++;
  q.r = *r;
  q.t_arrival = r->t_arrival >= 0.0 ? r->t_arrival : now_s(s);
  s->pending.push_back(q);
  s->st.submitted++;
  if (id) *id = q.id;
  return ELFEL_OK;
}

extern "C" int elfel_server_step(elfel_server* s, int32_t* active, int32_t* queued) {
  if (!s) return ELFEL_ERR_ARG;
  Ctx* c = &s->h->c;
  cudaSetDevice(c->device);
  const auto t = Clock::now();
  const int rc = s->batch ? step_batched(s, active) : step_plain(s, active);
  s->st.busy_seconds += std::chrono::duration<double>(Clock::now() - t).count();
  if (queued) *queued = (int32_t)s->pending.size();
  if (s->batch) {
    int64_t g = 0, k = 0;
    batch_counts(s->batch, &g, &k);
    s->st.graph_launches = g;
    s->st.solver_kernel_launches = k;
  }
  return rc;
}

extern "C" int elfel_server_poll(elfel_server* s, elfel_serve_result* out, int32_t cap, int32_t* n) {
  if (!s || !n || (cap > 0 && !out)) return ELFEL_ERR_ARG;
  const int k = std::min<int>((int)s->finished.size(), std::max(cap, 0));
  for (int i = 0; i < k; ++i) out[i] = s->finished[i];
  s->finished.erase(s->finished.begin(), s->finished.begin() + k);
  *n = k;
  return ELFEL_OK;
}

extern "C" int elfel_server_solution(elfel_server* s, int64_t id, double* T, int64_t n) {
  if (!s || !T) return ELFEL_ERR_ARG;
  Ctx* c = &s->h->c;
  auto it = s->solutions.find(id);
  if (it == s->solutions.end()) return fail(c, ELFEL_ERR_STATE, "solution: request %lld has none kept", (long long)id);
  if ((int64_t)it->second.size() != n)
    return fail(c, ELFEL_ERR_ARG, "solution: request %lld has %lld values", (long long)id,
                (long long)it->second.size());
  memcpy(T, it->second.data(), sizeof(double) * (size_t)n);
  s->solutions.erase(it);
  return ELFEL_OK;
}

extern "C" int elfel_server_stats_read(elfel_server* s, elfel_server_stats* out) {
  if (!s || !out) return ELFEL_ERR_ARG;
  *out = s->st;
  return ELFEL_OK;
}
