"""Benchmark of the GB300 element-assembly + sparse-solve path.

Default workload: the quadratic heat problem at scale -- unit square,
1000 x 1000 cells, 2 FEH1_T6 triangles per cell (2,000,000 elements,
4,004,001 nodes), interior vertices jittered by a seeded uniform +-0.2h
(midside nodes kept at edge midpoints), conductivity per element
log-uniform in [0.5, 2], Q = -6, Dirichlet T = 1 + x^2 + 2y^2 on the
boundary, 3-point rule.  Synthetic, seeded.

One step = one fused assembly of K and F (element integration + slot-map
reduction into the device CSC built once).  The JSON line reports
  value   elements assembled per second, inputs resident in HBM;
  e2e     the same metric through the C ABI from pinned host buffers:
          upload of mesh, DOF table and coefficients, pattern build,
          assembly, download of the CSC and F, every step;
  pcg     the solve of the same system to relative residual 1e-10 with
          FP64 Jacobi-PCG and with FP32 CG + FP64 residual replacement
          (one system, and the same in the batched engine), with the
          per-iteration roofline of both;
  serve   the serving stream: capacity, p50/p99 latency at three arrival
          rates, batched vs plain FP64 one request at a time;
  configs plane-strain T6 elasticity 1000 x 500 and the Taylor-Hood cavity
          600 x 600: assembly rate and both solver forms;
  roofline the dominant kernel's algorithmic bytes over its CUDA-event time
          against the measured HBM copy peak, with its measured DRAM traffic;
  cpu_baseline the CPU restatement of the reference path on the host cores;
  clocks  SM clocks and throttle reasons sampled during the timed region.

At N > 1 (torchrun, one rank per GPU) each rank assembles its own replica
and the line reports the sum; the pcg, serve and configs legs and the CPU
baseline run at N = 1 only.

``--impl reference`` times the CPU restatement of the reference path (the
oracle: element loop, COO triplets, SparseArrays.sparse semantics) on the
host cores instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CLOCK_WINDOW_S = 1.5
METRIC = "elems assembled/s; PCG time (FP32+refine vs FP64) at 1e-10; serve p50/p99"
UNIT = "elements/s"


def build_problem(E, N, seed=20261203, jit=0.2):
    mesh = E.T6block(1.0, 1.0, N, N)
    mesh = E.jitter(mesh, jit / N, seed=seed)
    fesp = E.FESpace(float, mesh, E.FEH1_T6())
    bn = E.boundary_nodes(mesh)
    x, y = mesh.xy[bn - 1, 0], mesh.xy[bn - 1, 1]
    E.setebc(fesp, 0, bn, 1, 1.0 + x ** 2 + 2.0 * y ** 2)
    E.numberdofs(fesp)
    rng = np.random.default_rng(seed + 1)
    kappa = np.exp(rng.uniform(np.log(0.5), np.log(2.0), mesh.nel))
    return mesh, fesp, kappa


def serving_workload(n, seed=20261204):
    """The serving stream: N log-uniform in [16, 512] (rounded), T3 or T6 with
    probability 1/2, kappa uniform in [0.5, 2], Q uniform in [-10, -1],
    Dirichlet T = 1 + x^2 + 2 y^2, unit square; seeded."""
    rng = np.random.default_rng(seed)
    N = np.rint(np.exp(rng.uniform(np.log(16.0), np.log(512.0), n))).astype(int)
    t6 = rng.random(n) < 0.5
    kappa = rng.uniform(0.5, 2.0, n)
    Q = rng.uniform(-10.0, -1.0, n)
    return [("T6" if t6[i] else "T3", int(N[i]), float(kappa[i]), float(Q[i])) for i in range(n)]


SERVE_MEM_BUDGET = 96 << 30  # device bytes a server may hold in resident systems


def run_stream(E, ctx, reqs, rate, method="pcg32_ir", batched=True, max_active=64, seed=7):
    """Serve reqs arriving as a Poisson stream of `rate` per second (rate None:
    all at t = 0, closed loop) on a fresh server; per-request latencies."""
    srv = E.HeatServer(method, batched=batched, max_active=max_active, rtol=1e-10, mem_budget=SERVE_MEM_BUDGET,
                       ctx=ctx)
    n = len(reqs)
    if rate:
        arr = np.cumsum(np.random.default_rng(seed).exponential(1.0 / rate, n))
    else:
        arr = np.zeros(n)
    t0 = srv.clock()
    done, i, active_sum, steps = [], 0, 0, 0
    while len(done) < n:
        now = srv.clock() - t0
        while i < n and arr[i] <= now:
            et, N, kap, Q = reqs[i]
            srv.submit(E.heat_request(et, N, kappa=kap, Q=Q, t_arrival=t0 + arr[i]))
            i += 1
        a, q = srv.step()
        active_sum += a
        steps += 1
        done.extend(srv.poll())
        if a == 0 and q == 0 and i < n and len(done) < n:
            time.sleep(max(0.0, min(arr[i] - (srv.clock() - t0), 0.01)))
    st = srv.stats()
    srv.close()
    lat = np.array([r["t_done"] - r["t_arrival"] for r in done])
    bad = [r for r in done if r["status"] != 0 or not r["converged"] or r["relres"] > 1e-10]
    span = max(r["t_done"] for r in done) - t0
    return {"requests": n, "offered_rate_per_s": rate, "solves_per_s": n / span, "makespan_s": span,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "mean_active": active_sum / max(steps, 1), "steps": steps,
            "failed": len(bad), "iterations_total": int(sum(r["iterations"] for r in done)),
            "elements_total": int(sum(r["nel"] for r in done)), "server": st}


def serve_bench(E, ctx, nreq, fracs, rate_sample):
    """The serving stream: capacity (closed loop, all nreq requests), the same
    requests solved one at a time by the plain FP64 path, and p50/p99 latency
    under Poisson arrivals at three rates (fractions of the measured capacity,
    printed as absolute rates) on the first rate_sample requests."""
    reqs = serving_workload(nreq)
    run_stream(E, ctx, reqs[:16], None)  # warm-up: graphs, autotuner records
    cap = run_stream(E, ctx, reqs, None)
    plain = run_stream(E, ctx, reqs, None, method="pcg64", batched=False)
    out = {"workload": f"{nreq} heat requests: unit square, N log-uniform [16,512], T3/T6 1:1, kappa U[0.5,2], "
                       f"Q U[-10,-1], T = 1 + x^2 + 2y^2 on the boundary, 3-point rule, FP32 CG + FP64 "
                       f"residual replacement to 1e-10 (seeded)",
           "closed_loop": cap, "capacity_solves_per_s": cap["solves_per_s"],
           "plain_fp64_one_at_a_time": {"sample": f"the same {nreq} requests, closed loop, FP64 Jacobi-PCG to 1e-10",
                                        "solves_per_s": plain["solves_per_s"], "makespan_s": plain["makespan_s"],
                                        "p50_ms": plain["p50_ms"], "p99_ms": plain["p99_ms"],
                                        "failed": plain["failed"]},
           "speedup_vs_plain": cap["solves_per_s"] / plain["solves_per_s"],
           "rate_sample": f"the first {min(rate_sample, nreq)} requests of the stream, Poisson arrivals",
           "rates": []}
    sub = reqs[:rate_sample]
    for f in fracs:
        r = run_stream(E, ctx, sub, f * cap["solves_per_s"])
        r["fraction_of_capacity"] = f
        out["rates"].append(r)
    out["rates_summary"] = [{"offered_per_s": r["offered_rate_per_s"], "achieved_per_s": r["solves_per_s"],
                             "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"]} for r in out["rates"]]
    return out


def build_elasticity(E, nx, ny, seed=20261205):
    """Plane strain on [0,2]x[0,1]: left edge clamped, unit traction on the right
    edge, body force per element uniform in [-0.1, 0.1]^2 (seeded)."""
    Lx, Ly = 2.0, 1.0
    mesh = E.T6block(Lx, Ly, nx, ny)
    fesp = E.FESpace(float, mesh, E.FEH1_T6(), 2)
    left = E.vselect(mesh.xy, [0.0, 0.0, 0.0, Ly], inflate=Lx / nx / 100)
    E.setebc(fesp, 0, left, 1, 0.0)
    E.setebc(fesp, 0, left, 2, 0.0)
    E.numberdofs(fesp)
    bforce = np.random.default_rng(seed).uniform(-0.1, 0.1, size=(mesh.nel, 2))
    be = E.boundary_edges(mesh)
    c = mesh.conn - 1
    le = be[:, 1] - 1
    a, b = c[be[:, 0] - 1, le], c[be[:, 0] - 1, (le + 1) % 3]
    right = be[(np.abs(mesh.xy[a, 0] - Lx) < 1e-12) & (np.abs(mesh.xy[b, 0] - Lx) < 1e-12)]
    return mesh, fesp, bforce, right


def build_cavity(E, N):
    """Lid-driven cavity, Taylor-Hood (vector T6 velocity, T3 pressure): u = (1, 0)
    on the top edge, 0 on the other walls, pressure pinned at one corner."""
    vmesh = E.T6block(1.0, 1.0, N, N)
    pmesh = E.T6toT3(vmesh)
    ufesp = E.FESpace(float, vmesh, E.FEH1_T6(), 2)
    pfesp = E.FESpace(float, pmesh, E.FEH1_T3(), 1)
    infl = 1.0 / N / 100
    for box in ([0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 0.0, 1.0], [1.0, 1.0, 0.0, 1.0]):
        vl = E.vselect(vmesh.xy, box, infl)
        E.setebc(ufesp, 0, vl, 1, 0.0)
        E.setebc(ufesp, 0, vl, 2, 0.0)
    vl = E.vselect(vmesh.xy, [0.0, 1.0, 1.0, 1.0], infl)
    E.setebc(ufesp, 0, vl, 1, 1.0)
    E.setebc(ufesp, 0, vl, 2, 0.0)
    E.setebc(pfesp, 0, 1, 1, 0.0)
    E.numberdofs([ufesp, pfesp])
    return vmesh, pmesh, ufesp, pfesp


def build_shape_problem(E, kind, N, seed=20261203, jit=0.2):
    """Heat on a Q4 block (N x N cells of the unit square) or a T4 block (N^3
    cubes of the unit cube, 6 tetrahedra each): vertices jittered +-jit*h,
    kappa log-uniform [0.5, 2] per element, T = 1 + x^2 + 2 y^2 on the boundary."""
    mesh = E.Q4block(1.0, 1.0, N, N) if kind == "Q4" else E.T4block(1.0, 1.0, 1.0, N, N, N)
    mesh = E.jitter(mesh, jit / N, seed=seed)
    fesp = E.FESpace(float, mesh, E.FEH1_Q4() if kind == "Q4" else E.FEH1_T4())
    bn = E.boundary_nodes(mesh)
    x, y = mesh.xy[bn - 1, 0], mesh.xy[bn - 1, 1]
    E.setebc(fesp, 0, bn, 1, 1.0 + x ** 2 + 2.0 * y ** 2)
    E.numberdofs(fesp)
    rng = np.random.default_rng(seed + 1)
    kappa = np.exp(rng.uniform(np.log(0.5), np.log(2.0), mesh.nel))
    return mesh, fesp, kappa


def problem_bench(E, ctx, args):
    """Elasticity (plane strain T6), Stokes (Taylor-Hood cavity) or heat on
    Q4 / T4 meshes at scale: fused assembly rate, and the FP64 vs
    FP32-refinement solves (one JSON line)."""
    out = problem_run(E, ctx, args.problem, args.n, args.steps, args.warmup, not args.no_pcg)
    print(json.dumps(out), flush=True)
    return 0


def problem_run(E, ctx, problem, n_cells, steps, warmup, solves):
    """The measurements of problem_bench as a dict: assembly (steps timed
    after warmup, L2 flushed between) and, with solves, both solver forms."""
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream())
    t0 = time.perf_counter()
    alg = None
    if problem in ("heat-q4", "heat-t4"):
        kind = "Q4" if problem == "heat-q4" else "T4"
        N = n_cells or (1414 if kind == "Q4" else 70)
        mesh, fesp, kappa = build_shape_problem(E, kind, N)
        n, nu = E.ndofs(fesp), E.nunknowns(fesp)
        qs = {"kind": "Gauss", "order": 2} if kind == "Q4" else {"npts": 1}
        elit, qpit = E.FEIterator(fesp), E.QPIterator(fesp, qs)
        am = E.start(E.SysmatAssemblerGPU(ctx), n, n)
        E.assemble_heat(am, elit, qpit, kappa, -6.0)  # set-up and coefficient upload
        step = lambda: am.heat(None, -6.0)
        methods, rtol = ("pcg64", "pcg32_ir"), 1e-10
        sd = mesh.sdim
        # compulsory bytes of one integration launch: conn 16 + coordinates + kappa 8 + records 14 x 8
        alg = {"integrate_heat": mesh.nel * (16 + 8 + 14 * 8) + mesh.nnodes * 8 * sd}
        work = (f"heat {kind} {'x'.join([str(N)] * (2 if kind == 'Q4' else 3))} ({mesh.nel} elements, {n} DOFs), "
                f"{'2x2 Gauss' if kind == 'Q4' else '1-point rule'}, fused K+F assembly, pattern reused")
        spaces = fesp
    elif problem == "elasticity":
        nx = n_cells or 1000
        mesh, fesp, bforce, right = build_elasticity(E, nx, nx // 2)
        n, nu = E.ndofs(fesp), E.nunknowns(fesp)
        elit, qpit = E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3})
        am = E.start(E.SysmatAssemblerGPU(ctx), n, n)
        step = lambda: E.assemble_elasticity(am, elit, qpit, 1.0, 0.3, True, bforce, right, (1.0, 0.0))
        methods, rtol = ("pcg64", "pcg32_ir"), 1e-10
        work = f"plane-strain elasticity T6 {nx}x{nx // 2} on [0,2]x[0,1] ({mesh.nel} elements, {n} DOFs)"
        spaces = fesp
    else:
        N = n_cells or 600
        vmesh, pmesh, ufesp, pfesp = build_cavity(E, N)
        n = E.ndofs(ufesp) + E.ndofs(pfesp)
        nu = E.nunknowns(ufesp) + E.nunknowns(pfesp)
        elit, pelit, qpit = E.FEIterator(ufesp), E.FEIterator(pfesp), E.QPIterator(ufesp, {"npts": 3})
        am = E.start(E.SysmatAssemblerGPU(ctx), n, n)
        step = lambda: E.assemble_stokes(am, elit, pelit, qpit, 1.0)
        methods, rtol = ("minres64", "minres32_ir"), 1e-8
        mesh = vmesh
        work = f"Stokes Taylor-Hood lid-driven cavity {N}x{N} ({vmesh.nel} elements, {n} DOFs)"
        spaces = [ufesp, pfesp]
    host_s = time.perf_counter() - t0
    step()  # set-up (tables, pattern) and a first assembly
    ctx.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        ctx.profile(True)
        evs = []
        for _ in range(steps):
            flush.zero_()  # L2 (129 MB) flushed between timed steps
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        phases = ctx.phases()
        ctx.profile(False)
    t_asm = sum(a.elapsed_time(b) for a, b in evs) / 1e3 / steps
    per = {k: (ms / cnt if cnt else 0.0) for k, (ms, cnt) in phases.items()}
    kernels = {k: {"ms_per_launch": v, "share": v / sum(per.values())} for k, v in per.items()}
    if alg:
        hbm, peak_kind = read_peaks()
        for k, b in alg.items():
            if per.get(k):
                kernels[k].update({"alg_bytes": b, "gbs": b / (per[k] * 1e-3) / 1e9,
                                   "frac": b / (per[k] * 1e-3) / 1e9 / hbm, "peak": hbm, "peak_kind": peak_kind})
    out = {"problem": problem, "workload": work, "elements": mesh.nel, "ndofs": n, "nunknowns": nu,
           "assembly_elements_per_s": mesh.nel / t_asm, "assembly_ms": t_asm * 1e3, "host_setup_s": host_s,
           "kernels": kernels, "l2": "256 MB buffer written between timed steps", "data": "synthetic (seeded)"}
    if solves:
        U0 = np.zeros(n)
        E.gathersysvec(U0, spaces)
        sols = {}
        for m in methods:
            U = U0.copy()
            st = am.solve(U, nu, None, method=m, rtol=rtol, maxit=500000)
            sols[m] = (st, U)
        (s64, U64), (s32, U32) = sols[methods[0]], sols[methods[1]]
        out.update({"rtol": rtol, methods[0]: s64, methods[1]: s32, "speedup": s64["seconds"] / s32["seconds"],
                    "fp32_vs_fp64_rel_err_max": float(np.abs(U32[:nu] - U64[:nu]).max() / np.abs(U64[:nu]).max())})
    del am
    return out


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.p = None
        self.window = None
        import tempfile

        self.path = os.path.join(tempfile.gettempdir(), f"elfel_clocks_{os.getpid()}.csv")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.Q}", "--format=csv,noheader",
                                       "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def mark(self, t0, t1):
        """The timed region, as datetime.now() values; samples outside it are dropped."""
        self.window = (t0, t1)

    def stop(self):
        import datetime

        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [s.strip() for s in line.split(",")]
                if len(parts) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                    if self.window and not (self.window[0] <= ts <= self.window[1]):
                        continue
                    sm.append(float(parts[2].split()[0]))
                    smax.append(float(parts[3].split()[0]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[6:10]):
                    if v.lower() == "active":
                        reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference_step(O, conn0, xy, ed, kappa, n):
    """One assembly of K and F by the CPU restatement of the reference path
    (test/test_heat.jl:35-71): the element loop (OpenMP over elements), the
    COO triplets of assemble! (column-major init!), SparseArrays.sparse
    semantics (single-threaded counting sorts, duplicates summed in append
    order) and the SysvecAssembler accumulation."""
    ke, fe = O.heat_element_matrices(6, 3, conn0, xy, kappa, -6.0)
    I, J, V = O.local_coo(ed, ed, ke)
    del ke
    K = O.sparse(I, J, V, n, n)
    del I, J, V
    F = O.vec_assemble(n, ed, fe)
    return K, F


def cpu_reference_rate(O, mesh, fesp, kappa, E, threads, steps, warmup=0):
    """Elements per second of cpu_reference_step on the whole mesh with
    `threads` OpenMP threads (mean over `steps` timed steps after `warmup`)."""
    ed = E.FEIterator(fesp).eldofs_table() - 1
    conn0 = np.ascontiguousarray(mesh.conn - 1)
    n = E.ndofs(fesp)
    O.set_threads(threads)
    times = []
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        K, F = cpu_reference_step(O, conn0, mesh.xy, ed, kappa, n)
        dt = time.perf_counter() - t0
        del K, F
        if k >= warmup:
            times.append(dt)
    t = sum(times) / len(times)
    return mesh.nel / t, t, len(times)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, dist, device="cpu"):
    """The largest x over all ranks (the step time every replica reports is the
    slowest one's); x itself without a process group."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def heat_config(N, ws):
    """The workload both arms report: the T6 heat problem on N x N cells."""
    nel, nnodes = 2 * N * N, (2 * N + 1) ** 2
    return {"workload": f"heat T6 {N}x{N} ({nel} elements, {nnodes} nodes), 3-point rule, "
                        f"fused K+F assembly, pattern reused",
            "elements": nel, "ndofs": nnodes, "nnz": 46 * N * N + 16 * N + 1,
            "l2": "256 MB buffer written between timed steps",
            "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU"}


def reference_arm(args):
    """The reference's own CPU path on the host cores, on the GPU arm's
    workload (the whole 2M-element mesh at the default size): every step is
    one complete assembly of K and F.  The steps run with all host threads in
    the element loop; one more step runs single-threaded, as the reference
    itself does (Julia, no threads), and is reported beside them."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__ as entry

    E = entry.package()
    O = entry.oracle()
    threads = os.cpu_count() or 1
    N = args.n or 1000
    mesh, fesp, kappa = build_problem(E, N)
    v, t, nsteps = cpu_reference_rate(O, mesh, fesp, kappa, E, threads, args.steps, args.warmup)
    v1, t1, _ = cpu_reference_rate(O, mesh, fesp, kappa, E, 1, 1)
    what = (f"T6 heat {N}x{N} ({mesh.nel} elements), the whole mesh every step: element loop + COO triplets + "
            f"sparse() (single-threaded) + vector assembly")
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
           "config": heat_config(N, ws),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"{what}; element loop on {threads} threads; mean of {nsteps} steps",
                            "single_thread": {"value": v1, "unit": UNIT, "cores": 1, "ms_per_step": t1 * 1e3,
                                              "sample": f"{what}; one thread throughout; one step"}},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 300 on the GPU; 10 for the reference arm, whose every step is a "
                         "full CPU assembly of seconds)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=None, help="cells per side (heat, elasticity: 1000; Stokes: 600)")
    ap.add_argument("--problem", default="heat", choices=["heat", "elasticity", "stokes", "heat-q4", "heat-t4"],
                    help="heat: the contract line; elasticity / stokes / heat-q4 / heat-t4: assembly rate and "
                         "solves at scale")
    ap.add_argument("--no-pcg", action="store_true")
    ap.add_argument("--pcg-methods", default="pcg64,pcg32_ir", help="solves to run, in order")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=2, help="full-size CPU reference steps of the cpu_baseline")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the elasticity 1000x500 and Stokes 600x600 legs (assembly and both solves)")
    ap.add_argument("--serve-requests", type=int, default=4096, help="requests of the serving stream")
    ap.add_argument("--serve-rates", default="0.5,0.7,0.9", help="arrival rates as fractions of the capacity")
    ap.add_argument("--serve-rate-sample", type=int, default=1024,
                    help="requests (from the start of the stream) of each Poisson-arrival pass")
    ap.add_argument("--probe-rates", action="store_true", help="print the device's FP64/FP32 FMA rates and exit")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 10 if args.impl == "reference" else 300
    if args.impl == "reference":
        return reference_arm(args)
    assert args.warmup >= 3 or os.environ.get("ELFEL_BENCH_ALLOW_FEW_WARMUP"), "at least 3 warm-up steps"

    import torch

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import __graft_entry__ as entry

    E = entry.package()
    if rank == 0:
        E.build()  # incremental: a no-op when the library is current
    if dist:
        dist.barrier()
    E._native.load()
    ctx = E.Context(local)
    rates = {"fp64_tflops": ctx.fma_rate(64), "fp32_tflops": ctx.fma_rate(32)}
    if args.probe_rates:
        if rank == 0:
            print(json.dumps(rates), flush=True)
        ctx.close()
        return 0
    if args.problem != "heat":
        rc = problem_bench(E, ctx, args) if rank == 0 else 0
        ctx.close()
        return rc
    stream = torch.cuda.ExternalStream(ctx.stream())
    N = args.n or 1000
    t_setup0 = time.perf_counter()
    mesh, fesp, kappa = build_problem(E, N)
    host_setup_s = time.perf_counter() - t_setup0
    nel = mesh.nel
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    elit = E.FEIterator(fesp)
    qpit = E.QPIterator(fesp, {"kind": "default", "npts": 3})

    # --- device-resident assembly (value) ---------------------------------
    am = E.start(E.SysmatAssemblerGPU(ctx), n, n)
    ctx.profile(True)
    t0 = time.perf_counter()
    am.setup(E._native.ELFEL_HEAT, elit, qpit)
    ctx.synchronize()
    pattern_s = time.perf_counter() - t0
    setup_phases = ctx.phases()
    am.heat(kappa, -6.0)  # uploads the coefficients once
    ctx.synchronize()
    ctx.profile(False)
    flush =torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    import datetime

    clocks = Clocks(local)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            am.heat(None, -6.0)
        torch.cuda.synchronize()
        time.sleep(0.3)  # let the sampler start
        if dist:
            dist.barrier()
        ctx.profile(True)
        evs = []
        dt0 = datetime.datetime.now()
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()  # L2 (129 MB) flushed between timed steps
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            am.heat(None, -6.0)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        ctx.profile(False)
        # the timed steps take milliseconds, shorter than the sampler's period:
        # the same steps continue, untimed, for CLOCK_WINDOW_S so that the
        # clock record covers the timed steps and this continuation
        t_ext = time.perf_counter()
        ext = 0
        while time.perf_counter() - t_ext < CLOCK_WINDOW_S:
            for _ in range(50):
                flush.zero_()
                am.heat(None, -6.0)
            torch.cuda.synchronize()
            ext += 50
        clocks.mark(dt0, datetime.datetime.now())
        clk = clocks.stop()
        clk["window"] = f"the {args.steps} timed steps and {ext} more of the same steps right after them"
    phases = ctx.phases()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    t_step = sum(step_ms) / len(step_ms) / 1e3
    t_step = max_over_ranks(t_step, dist, f"cuda:{local}" if torch.cuda.is_available() else "cpu")
    value = ws * nel / t_step

    # --- roofline of the dominant kernel (live CUDA events) ---------------
    hbm, peak_kind = read_peaks()
    nslots = nel * 36
    nnz_est = 46 * N * N + 16 * N + 1
    per = {k: (ms / cnt if cnt else 0.0) for k, (ms, cnt) in phases.items()}
    # without a reduce_F phase the integration kernel added the load vector
    # itself (midside DOFs read, the vector written) instead of writing records
    f_direct = "reduce_F" not in per
    ntiles, nprog, nfb, nruns = am.tile_stats()
    tiles = ntiles > 0  # a resident pattern's assemblies take the tile reduction (8 bases per element)
    design = {  # bytes each kernel itself must move per launch, as designed (its own inputs and outputs)
        "integrate_heat": nel * 6 * 4 + mesh.nnodes * 16 + nel * 8 + nel * (8 if tiles else 21) * 8 +
                          (nel * 3 * 4 + n * 8 if f_direct else nel * 6 * 8),
        # tiles: the bases (64 B per element, read once from DRAM) and the values; the
        # programs stay in L2. Contributor lists: cptr, contributor indices, records, values
        "reduce_K": (nel * 8 * 8 + nnz_est * 8) if tiles else
                    ((nnz_est + 1) * 4 + nslots * 4 + nel * 21 * 8 + nnz_est * 8),
        "reduce_F": (n + 1) * 8 + (n + 1) * 4 + nel * 6 * 4 + nel * 6 * 8 + n * 8,
    }
    dom = max(per, key=per.get)
    # algorithmic bytes of one assembly, the roofline's numerator: connectivity
    # (6 x int32 per element) + node coordinates (16 B per node) + conductivity
    # (8 B per element) + K values (8 B per nonzero) + F (8 B per DOF), each
    # read or written once -- 264 B per element, 528.2 MB at 2M elements
    asm_bytes = nel * 6 * 4 + mesh.nnodes * 16 + nel * 8 + nnz_est * 8 + n * 8
    kernel_rows = {k: {"ms_per_launch": per[k], "share": per[k] / sum(per.values()),
                       "design_bytes": design.get(k),
                       "design_gbs": (design[k] / (per[k] * 1e-3) / 1e9) if k in design and per[k] else None}
                   for k in per}
    # DRAM traffic of one launch of each kernel (dram__bytes_read.sum + dram__bytes_write.sum)
    # measured with ncu on the 700 x 700 case of this workload (980,000 elements), scaled by
    # the element count; writes still dirty in L2 when a kernel ends are not counted.
    # Tile path: heat_t6_bases_k 86.67 + 28.99 MB, tile_run_k 66.04 + 126.17 MB.
    # Contributor-list path: heat_t6s_k<2, 1> 86.84 + 121.46 MB (<2, 0> 47.34 + 151.06 MB),
    # reduce_win_k 426.95 + 155.19 MB, reduce_row0_dense_k 94.18 + 8.28 MB.
    if tiles:
        TRAFFIC_PER_ELEMENT = {"integrate_heat": (86.668288e6 + 28.988672e6) / 980000,
                               "reduce_K": (66.036480e6 + 126.165248e6) / 980000}
    else:
        TRAFFIC_PER_ELEMENT = {"integrate_heat": ((86.844672e6 + 121.461504e6) if f_direct else
                                                  (47.341056e6 + 151.063040e6)) / 980000,
                               "reduce_K": (426.946560e6 + 155.187456e6) / 980000,
                               "reduce_F": (94.176768e6 + 8.283392e6) / 980000}
    traffic = TRAFFIC_PER_ELEMENT[dom] * nel if dom in TRAFFIC_PER_ELEMENT else None
    for k, row in kernel_rows.items():
        row["traffic"] = TRAFFIC_PER_ELEMENT[k] * nel if k in TRAFFIC_PER_ELEMENT else None
    ach = asm_bytes / (per[dom] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": traffic, "kernel": dom, "peak_kind": peak_kind, "alg_bytes": asm_bytes,
                "alg_bytes_what": "one assembly: connectivity + coordinates + conductivity + K values + F, once each "
                                  "(264 B/element); achieved = these bytes / the dominant kernel's mean CUDA-event "
                                  "time",
                "traffic_source": "ncu DRAM bytes of the kernel at 980,000 elements, scaled per element "
                                  "(profiles/tile_run_T6_700.md)",
                "assembly": {"alg_bytes": asm_bytes, "achieved": asm_bytes / t_step / 1e9,
                             "frac": asm_bytes / t_step / 1e9 / hbm, "what": "the same bytes / the whole step"},
                "kernels": kernel_rows}

    roofline["tile_plan"] = {"tiles": ntiles, "programs": nprog, "fallback_tiles": nfb, "runs": nruns}

    # --- e2e through the C ABI from pinned host buffers -------------------
    conn_h = torch.from_numpy(np.ascontiguousarray(mesh.conn)).pin_memory()
    xy_h = torch.from_numpy(np.ascontiguousarray(mesh.xy)).pin_memory()
    dofs_h = torch.from_numpy(elit.eldofs_table()).pin_memory()
    kap_h = torch.from_numpy(kappa).pin_memory()
    nnz_dev = int(46 * N * N + 16 * N + 1)
    colptr_h = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    rowval_h = torch.empty(nnz_dev, dtype=torch.int64).pin_memory()
    nzval_h = torch.empty(nnz_dev, dtype=torch.float64).pin_memory()
    F_h = torch.empty(n, dtype=torch.float64).pin_memory()
    import ctypes

    N_ = E._native
    pc = N_.f64(qpit.quadr.param_coords)
    w = N_.f64(qpit.quadr.weights)

    def as_p(t, typ):
        return ctypes.cast(ctypes.c_void_p(t.data_ptr()), typ)

    sp = N_.Space(6, 1, nel, mesh.nnodes, as_p(conn_h, N_._i64p), as_p(xy_h, N_._dp), as_p(dofs_h, N_._i64p))
    desc = N_.FusedDesc(N_.ELFEL_HEAT, 3, N_.ptr(pc), N_.ptr(w), n, sp, N_.Space())
    lib = ctx.lib
    hm = ctypes.c_void_p()
    ctx.check(lib.elfel_sysmat_create(ctx.h, ctypes.byref(hm)))

    def e2e_step():
        ctx.check(lib.elfel_fused_setup(hm, ctypes.byref(desc)))
        ctx.check(lib.elfel_fused_heat(hm, as_p(kap_h, N_._dp), -6.0))
        ctx.check(lib.elfel_sysmat_csc(hm, as_p(colptr_h, N_._i64p), as_p(rowval_h, N_._i64p), as_p(nzval_h, N_._dp)))
        ctx.check(lib.elfel_sysmat_rhs(hm, as_p(F_h, N_._dp)))

    e2e_steps = max(2, min(args.steps, 5))
    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    lib.elfel_sysmat_destroy(hm)
    h2d = conn_h.numel() * 8 + xy_h.numel() * 8 + dofs_h.numel() * 8 + kap_h.numel() * 8 + pc.nbytes + w.nbytes
    d2h = colptr_h.numel() * 8 + rowval_h.numel() * 8 + nzval_h.numel() * 8 + F_h.numel() * 8
    e2e = {"value": ws * nel / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "ms_per_step": t_e2e * 1e3,
           "what": "C-ABI fused_setup (H2D mesh+eldofs, device pattern build) + fused_heat (H2D kappa) + CSC/F D2H"}
    assert int(colptr_h[-1]) == nnz_dev + 1  # pattern size of the uniform T6 block

    # The solver, serving and configuration legs and the CPU baseline are
    # single-GPU measurements: they run at N = 1 only (N > 1 times the
    # assembly replicas alone).
    single = ws == 1

    # --- PCG: FP64 vs FP32 + FP64 refinement, to 1e-10 ---------------------
    pcg = None
    if not args.no_pcg and single:
        T0 = np.zeros(n)
        E.gathersysvec(T0, fesp)
        res = {}
        for method in args.pcg_methods.split(","):
            T = T0.copy()
            torch.cuda.synchronize()
            st = am.solve(T, nu, None, method=method, rtol=1e-10)
            res[method] = (st, T)
        pcg = {"rtol": 1e-10}
        for method, key in (("pcg64", "fp64"), ("pcg32_ir", "fp32_ir")):
            if method in res:
                pcg[key] = res[method][0]
        if "pcg64" in res and "pcg32_ir" in res:
            st64, T64 = res["pcg64"]
            st32, T32 = res["pcg32_ir"]
            pcg["speedup"] = st64["seconds"] / st32["seconds"]
            pcg["fp32_vs_fp64_rel_err_max"] = float(np.abs(T32[:nu] - T64[:nu]).max() / np.abs(T64[:nu]).max())
        # per-iteration roofline: algorithmic bytes of one iteration on the free-free block
        # (FP64: values 8 + column index 4 per nonzero, row pointer 4 and ~10 vector
        # accesses of 8 per unknown; FP32 inner iteration: 4 + 4 per nonzero, ~10 vector
        # accesses of 4 per unknown) x iterations / solve time
        cp1 = colptr_h.numpy()
        rv1 = rowval_h.numpy()[: int(cp1[nu]) - 1]
        nnz_ff = int(np.count_nonzero(rv1 <= nu))
        per_it = {"fp64": nnz_ff * 12 + nu * 4 + 10 * nu * 8, "fp32_ir": nnz_ff * 8 + 10 * nu * 4}
        pcg["roofline"] = {"nnz_ff": nnz_ff, "nu": nu, "peak": hbm, "unit": "GB/s",
                           "what": "iterations x algorithmic bytes per iteration / solve time (FP32: the inner "
                                   "iterations; the FP64 residual replacements are not counted)"}
        for key in ("fp64", "fp32_ir"):
            if key in pcg:
                gbs = pcg[key]["iterations"] * per_it[key] / pcg[key]["seconds"] / 1e9
                pcg["roofline"][key] = {"bytes_per_iteration": per_it[key], "achieved": gbs, "frac": gbs / hbm}
        if "pcg32_ir" in res:
            # the batched form with this one system: per-tile kernels, device-side replacement
            b = E.BatchSolver("pcg32_ir", capacity=1, ctx=ctx)
            torch.cuda.synchronize()
            tb0 = time.perf_counter()
            s = b.add(am, T0, nu, rtol=1e-10)
            Tb, stb = b.run(graphs=8)[s]
            tb = time.perf_counter() - tb0
            b.close()
            pcg["fp32_ir_batched"] = dict(stb, wall_s=tb)
            if "pcg64" in res:
                pcg["speedup_batched"] = res["pcg64"][0]["seconds"] / tb
                pcg["batched_vs_fp64_rel_err_max"] = float(np.abs(Tb[:nu] - T64[:nu]).max() / np.abs(T64[:nu]).max())

    # --- serving stream: p50/p99 at three arrival rates ------------------
    serve = None
    if not args.no_serve and single:
        fr = [float(x) for x in args.serve_rates.split(",") if x]
        serve = serve_bench(E, ctx, args.serve_requests, fr, args.serve_rate_sample)
        serve["tuning"] = [t for t, _ in ctx.tuning()]

    # --- the other configurations: plane-strain elasticity 1000 x 500 and the
    # Taylor-Hood cavity 600 x 600 (assembly, FP64 and FP32-refinement solves)
    configs = None
    if not args.no_configs and single:
        configs = {prob: problem_run(E, ctx, prob, ncell, 5, 3, not args.no_pcg)
                   for prob, ncell in (("elasticity", 1000), ("stokes", 600))}

    # --- CPU baseline (oracle restatement on the host cores) --------------
    cpu = None
    if single and not args.no_cpu:
        O = entry.oracle()
        threads = os.cpu_count() or 1
        rate, tper, reps = cpu_reference_rate(O, mesh, fesp, kappa, E, threads, args.cpu_steps)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"T6 heat {N}x{N} ({nel} elements), the whole mesh: element loop ({threads} threads) + "
                         f"COO triplets + sparse() (single-threaded) + vector assembly; mean of {reps} steps, "
                         f"{tper:.3f} s each"}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (seeded T6 mesh, jitter 0.2h, kappa log-uniform [0.5,2])",
           "config": heat_config(N, ws),
           "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": (2 if f_direct else 3) * args.steps, "clocks": clk,
           "pcg": pcg, "serve": serve, "configs": configs, "fma_rates": rates, "pattern_build_s": pattern_s, "setup_phases_ms": {k: v[0] for k, v in setup_phases.items()},
           "wall_s_timed": wall, "host_mesh_setup_s": host_setup_s}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    del am
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
