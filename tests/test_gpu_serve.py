"""Device block meshes and the serving loop (GPU).

Bars:
  * device-generated block meshes equal the host generators and the host
    DOF numbering bit for bit (connectivity, coordinates, element DOFs,
    Dirichlet vector), and so do the assembled K and F;
  * every served request converges to rtol and equals, bit for bit, the same
    problem solved alone in the batched solver -- whatever else was running
    (continuous batching changes no result);
  * the plain one-at-a-time mode agrees with the batched mode within
    ERR_TOL, and T6 reproduces the exact quadratic within QUAD_TOL.
"""
import numpy as np
import pytest

from problems import heat_space

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-8
QUAD_TOL = 1e-8
COEF = (1.0, 0.0, 0.0, 1.0, 0.0, 2.0)  # T = 1 + x^2 + 2 y^2, exact for Q = -6, kappa = 1


def host_problem(E, etype, nx, ny, lx, ly, orient):
    blk = E.T3block if etype == "T3" else E.T6block
    mesh = blk(lx, ly, nx, ny, orientation=orient)
    fesp = heat_space(E, mesh, E.FEH1_T3() if etype == "T3" else E.FEH1_T6())
    T = np.zeros(E.ndofs(fesp))
    E.gathersysvec(T, fesp)
    return mesh, fesp, T


@pytest.mark.parametrize("etype,nx,ny,lx,ly,orient", [("T3", 7, 5, 1.0, 1.0, "a"), ("T3", 6, 6, 2.0, 0.5, "alternate"),
                                                      ("T6", 4, 3, 1.0, 1.0, "a"), ("T6", 5, 5, 0.7, 1.3, "alternate"),
                                                      ("T3", 1, 1, 1.0, 1.0, "a")])
def test_block_tables_match_host(E, gpu, etype, nx, ny, lx, ly, orient):
    mesh, fesp, T0 = host_problem(E, etype, nx, ny, lx, ly, orient)
    am = E.SysmatAssemblerGPU()
    n, nu = am.setup_block(etype, nx, ny, lx, ly, orient)
    assert n == E.ndofs(fesp) and nu == E.nunknowns(fesp)
    conn, xy, dofs = am.tables()
    assert np.array_equal(conn, mesh.conn)
    assert np.array_equal(xy, mesh.xy)
    assert np.array_equal(dofs, E.FEIterator(fesp).eldofs_table())
    assert np.array_equal(am.block_dirichlet(COEF), T0)


def test_block_assembly_matches_host_tables(E, gpu):
    mesh, fesp, _ = host_problem(E, "T6", 9, 7, 1.0, 1.0, "alternate")
    n = E.ndofs(fesp)
    a1 = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(a1, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.3, -4.0)
    a2 = E.SysmatAssemblerGPU()
    a2.setup_block("T6", 9, 7, 1.0, 1.0, "alternate")
    a2.heat(1.3, -4.0)
    K1, K2 = a1.csc(), a2.csc()
    assert np.array_equal(K1.indptr, K2.indptr) and np.array_equal(K1.indices, K2.indices)
    assert np.array_equal(K1.data, K2.data)
    assert np.array_equal(a1.rhs(), a2.rhs())


REQS = [("T3", 20, 1.0, -6.0), ("T6", 12, 1.7, -3.0), ("T3", 57, 0.6, -9.5), ("T6", 33, 1.0, -6.0),
        ("T3", 16, 1.2, -1.0), ("T6", 12, 0.8, -7.0), ("T3", 90, 1.9, -2.0), ("T6", 5, 1.0, -6.0)]


def alone_in_batch(E, etype, N, kappa, Q, method="pcg32_ir"):
    am = E.SysmatAssemblerGPU()
    n, nu = am.setup_block(etype, N, N)
    am.heat(kappa, Q)
    T = am.block_dirichlet(COEF)
    b = E.BatchSolver(method, capacity=1)
    s = b.add(am, T, nu, rtol=1e-10)
    out = b.run()
    b.close()
    return out[s][0]


def test_served_equals_alone(E, gpu):
    srv = E.HeatServer("pcg32_ir", max_active=4, rtol=1e-10)
    ids = {}
    for etype, N, kappa, Q in REQS:
        ids[srv.submit(E.heat_request(etype, N, kappa=kappa, Q=Q, keep_solution=True))] = (etype, N, kappa, Q)
    res = srv.drain()
    assert len(res) == len(REQS)
    for r in res:
        assert r["status"] == 0 and r["converged"] and r["relres"] <= 1e-10, r
        assert r["t_arrival"] <= r["t_admit"] <= r["t_done"]
        T = srv.solution(r["id"])
        etype, N, kappa, Q = ids[r["id"]]
        assert np.array_equal(T, alone_in_batch(E, etype, N, kappa, Q)), (etype, N)
    st = srv.stats()
    assert st["completed"] == len(REQS) and st["systems_reused"] >= 1  # the two T6 N=12 requests share a mesh
    srv.close()


def test_large_wave_autotuned_assembly(E, gpu):
    """A wave above the tuner's threshold: every candidate CTA size of the
    batched integration runs, and the result is still the alone result."""
    srv = E.HeatServer("pcg32_ir", max_active=4)
    rid = srv.submit(E.heat_request("T6", 190, kappa=1.1, Q=-5.0, keep_solution=True))
    srv.submit(E.heat_request("T6", 7, kappa=0.9, Q=-2.0))
    res = {r["id"]: r for r in srv.drain()}
    assert res[rid]["converged"]
    assert np.array_equal(srv.solution(rid), alone_in_batch(E, "T6", 190, 1.1, -5.0))
    assert any(line.startswith("heat_batch_T6") for line, _ in gpu.tuning())
    srv.close()


def test_exact_quadratic_and_plain_mode(E, gpu):
    srvb = E.HeatServer("pcg32_ir", max_active=8)
    srvp = E.HeatServer("pcg64", batched=False)
    for s in (srvb, srvp):
        s.submit(E.heat_request("T6", 24, keep_solution=True))
        s.submit(E.heat_request("T3", 40, orientation="alternate", keep_solution=True))
    rb = sorted(srvb.drain(), key=lambda r: r["id"])
    rp = sorted(srvp.drain(), key=lambda r: r["id"])
    Tb = [srvb.solution(r["id"]) for r in rb]
    Tp = [srvp.solution(r["id"]) for r in rp]
    for a, b in zip(Tb, Tp):
        assert np.abs(a - b).max() / np.abs(b).max() < ERR_TOL
    # T6 reproduces the quadratic T = 1 + x^2 + 2 y^2 exactly
    mesh, fesp, _ = host_problem(E, "T6", 24, 24, 1.0, 1.0, "a")
    ex = 1.0 + mesh.xy[:, 0] ** 2 + 2.0 * mesh.xy[:, 1] ** 2
    dof = fesp.field.dofnums[:, 0] - 1
    assert np.abs(Tb[0][dof] - ex).max() < QUAD_TOL
    srvb.close()
    srvp.close()


def test_memory_budget_evicts_and_waits(E, gpu):
    """A budget that holds about two systems: requests wait for memory, idle
    systems are evicted, and every request still completes correctly."""
    srv = E.HeatServer("pcg32_ir", max_active=8, mem_budget=40 << 20)
    sizes = [("T6", 60), ("T3", 120), ("T6", 61), ("T3", 121), ("T6", 62)]
    for etype, N in sizes:
        srv.submit(E.heat_request(etype, N))
    res = srv.drain()
    st = srv.stats()
    assert len(res) == len(sizes) and all(r["status"] == 0 and r["converged"] for r in res)
    assert st["systems_evicted"] >= 1
    assert st["resident_bytes"] <= 40 << 20
    srv.close()
