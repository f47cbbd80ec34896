"""Device solves against the oracle's direct solve (GPU).

Each solve must reach the requested relative residual ||b - K x|| / ||b||
(computed in FP64 on the device) and match the oracle's SuperLU solution of
the same lifted system within ERR_TOL (relative, max norm).
"""
import numpy as np
import pytest

from problems import elasticity_setup, heat_oracle, heat_space, stokes_errors, stokes_oracle_K, stokes_setup

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-8  # solution error vs the FP64 direct solve at rtol = 1e-10..1e-12


def heat_system(E, etype, N, orientation="a", jit=0.0, kappa=None, npts=3):
    blk = E.T3block if etype == "T3" else E.T6block
    mesh = blk(1.0, 1.0, N, N, orientation=orientation)
    if jit:
        mesh = E.jitter(mesh, jit / N, seed=5)
    fesp = heat_space(E, mesh, E.FEH1_T3() if etype == "T3" else E.FEH1_T6())
    n = E.ndofs(fesp)
    if kappa is None:
        rng = np.random.default_rng(9)
        kappa = np.exp(rng.uniform(np.log(0.5), np.log(2.0), mesh.nel))
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": npts}), kappa, -6.0)
    return mesh, fesp, am, kappa


def test_heat_t3_golden_on_device(E, gpu, golden):
    """test/test_heat.jl:89-111 end to end on the device: golden T vector, exact nodal values."""
    g = golden("heat_t3.json")
    for method in ("pcg64", "pcg32_ir"):
        # a fresh space per run: scattersysvec! leaves the solution in the free
        # DOF values, and solve! would then solve for a correction
        mesh = E.T3block(g["A"], g["A"], g["N"], g["N"])
        fesp = heat_space(E, mesh, E.FEH1_T3())
        n, nu = E.ndofs(fesp), E.nunknowns(fesp)
        am = E.start(E.SysmatAssemblerGPU(), n, n)
        E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"kind": "default"}), g["kappa"], g["Q"])
        T = np.zeros(n)
        E.gathersysvec(T, fesp)
        st = E.solve(T, am, None, nu, method=method, rtol=1e-12)
        assert st["converged"]
        assert np.allclose(T, g["T"], rtol=1e-9, atol=1e-12)
        E.scattersysvec(fesp, T)
        vals = E.makeattribute(fesp, "T", 1)[:, 0]
        ex = 1.0 + mesh.xy[:, 0] ** 2 + 2 * mesh.xy[:, 1] ** 2
        assert np.mean(np.abs(vals - ex)) <= g["mean_nodal_error_max"]


@pytest.mark.parametrize("method", ["pcg64", "pcg32_ir"])
@pytest.mark.parametrize("etype,N,orient,jit", [("T3", 100, "alternate", 0.0), ("T6", 40, "a", 0.2),
                                                ("T3", 60, "a", 0.1), ("T6", 25, "alternate", 0.0)])
def test_heat_solve_vs_direct(E, O, gpu, method, etype, N, orient, jit):
    mesh, fesp, am, kappa = heat_system(E, etype, N, orient, jit)
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, kappa, -6.0)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    T0 = O.solve_lifted(K0, F0, T.copy(), nu)
    st = E.solve(T, am, None, nu, method=method, rtol=1e-11)
    assert st["converged"] and st["relres"] <= 1e-11
    assert np.abs(T - T0).max() / np.abs(T0).max() < ERR_TOL


def test_high_contrast_reaches_tolerance(E, O, gpu):
    """Conductivity over eight decades at rtol 1e-12: the FP64 recurrence can
    claim convergence before the true residual gets there; the one-system and
    the batched FP64 PCG check the true residual and continue, so both end at
    rtol (true FP64 residual) and at the direct solution."""
    rng = np.random.default_rng(17)
    mesh, fesp, am, kappa = heat_system(E, "T3", 64, "alternate", 0.0,
                                        kappa=np.exp(rng.uniform(np.log(1e-4), np.log(1e4), 2 * 64 * 64)))
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, kappa, -6.0)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    T0 = O.solve_lifted(K0, F0, T.copy(), nu)
    T1 = T.copy()
    st = E.solve(T1, am, None, nu, method="pcg64", rtol=1e-12, maxit=200000)
    assert st["converged"] and st["relres"] <= 1e-12
    b = E.BatchSolver("pcg64", capacity=1)
    s = b.add(am, T, nu, rtol=1e-12, maxit=200000)
    T2, st2 = b.run()[s]
    b.close()
    assert st2["converged"] and st2["relres"] <= 1e-12
    for Tx in (T1, T2):  # error bar of this conditioning (contrast 1e8): 1e-4
        assert np.abs(Tx - T0).max() / np.abs(T0).max() < 1e-4


def test_heat_t3_exact_config0(E, gpu):
    """The 100 x 100 T3 heat problem (uniform diagonals) reproduces the exact quadratic."""
    mesh, fesp, am, _ = heat_system(E, "T3", 100, kappa=1.0)
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    st = E.solve(T, am, None, nu, method="pcg32_ir", rtol=1e-12)
    assert st["converged"]
    ex = 1.0 + mesh.xy[:, 0] ** 2 + 2 * mesh.xy[:, 1] ** 2
    assert np.mean(np.abs(T[fesp.field.dofnums[:, 0] - 1] - ex)) <= 1e-9


def test_solve_with_host_rhs_and_nonzero_free_start(E, O, gpu):
    """solve! semantics with F given and nonzero free entries of T (test/test_heat.jl:73-76)."""
    mesh, fesp, am, kappa = heat_system(E, "T6", 12)
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, kappa, -6.0)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    T[:nu] = 0.25
    F = F0 * 0.5
    T0 = O.solve_lifted(K0, F, T.copy(), nu)
    E.solve(T, am, F, nu, method="pcg64", rtol=1e-12)
    assert np.abs(T - T0).max() / np.abs(T0).max() < ERR_TOL


@pytest.mark.parametrize("method", ["pcg64", "pcg32_ir"])
def test_generic_matrix_wide_columns(E, O, gpu, method):
    """A host CSC with randomly renumbered DOFs (column deltas beyond 16 bits -> 32-bit
    column path), some data DOFs, solved through solve!(T, K, F, nu)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(12)
    m = 200
    L1 = sp.diags([-np.ones(m - 1), 2.0 * np.ones(m), -np.ones(m - 1)], [-1, 0, 1])
    A = (sp.kron(sp.eye(m), L1) + sp.kron(L1, sp.eye(m))).tocsr()  # 40,000 unknowns
    p = rng.permutation(A.shape[0])
    A = A[p][:, p].tocsc()
    n = A.shape[0]
    nu = n - 500
    F = rng.standard_normal(n)
    T = np.zeros(n)
    T[nu:] = rng.standard_normal(n - nu)
    T0 = O.solve_lifted(A, F, T.copy(), nu)
    st = E.solve(T, A, F, nu, method=method, rtol=1e-11)
    assert st["converged"]
    assert np.abs(T - T0).max() / np.abs(T0).max() < ERR_TOL


def test_correction_solve_tiny_rhs(E, gpu):
    """solve! from an already converged T: the lifted rhs is roundoff (~1e-15);
    the FP32 refinement must still reach the relative tolerance (no FP32 underflow)."""
    mesh, fesp, am, _ = heat_system(E, "T3", 8, kappa=1.0)
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    E.solve(T, am, None, nu, method="pcg64", rtol=1e-13)
    for method in ("pcg64", "pcg32_ir"):
        T2 = T.copy()
        st = E.solve(T2, am, None, nu, method=method, rtol=1e-6)
        assert st["converged"]
        assert np.abs(T2[:nu]).max() < 1e-12  # the correction of a converged solution


def test_not_converged_reports(E, gpu):
    mesh, fesp, am, _ = heat_system(E, "T6", 30)
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    with pytest.raises(E.NotConverged):
        E.solve(T, am, None, nu, method="pcg64", rtol=1e-12, maxit=5)


@pytest.mark.parametrize("method", ["pcg64", "pcg32_ir"])
def test_elasticity_solve(E, O, gpu, method):
    mesh, fesp, bforce, right = elasticity_setup(E, 24, 12)
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_elasticity(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.0, 0.3, True, bforce, right,
                          (1.0, 0.0))
    K, F = E.finish(am), am.rhs()
    U = np.zeros(n)
    E.gathersysvec(U, fesp)
    U0 = O.solve_lifted(K, F, U.copy(), nu)
    st = E.solve(U, am, None, nu, method=method, rtol=1e-11)
    assert st["converged"]
    assert np.abs(U - U0).max() / np.abs(U0).max() < ERR_TOL


@pytest.mark.parametrize("method", ["minres64", "minres32_ir"])
def test_stokes_veclap_golden_on_device(E, O, gpu, golden, method):
    """test/test_stokes.jl:777-780 with device assembly and MINRES."""
    g = golden("stokes.json")["veclap_th_errors"]
    vmesh, pmesh, ufesp, pfesp = stokes_setup(E, g["N"])
    n = E.ndofs(ufesp) + E.ndofs(pfesp)
    nu = E.nunknowns(ufesp) + E.nunknowns(pfesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_stokes(am, E.FEIterator(ufesp), E.FEIterator(pfesp), E.QPIterator(ufesp, {"npts": 3}), 1.0)
    U = np.zeros(n)
    E.gathersysvec(U, [ufesp, pfesp])
    st = E.solve(U, am, None, nu, method=method, rtol=1e-12, maxit=20000)
    assert st["converged"]
    ep, ev = stokes_errors(O, vmesh, pmesh, ufesp, pfesp, U)
    assert np.allclose([ep, ev], g["ep_ev"], rtol=1e-7)


@pytest.mark.parametrize("method", ["minres64", "minres32_ir"])
def test_stokes_cavity_vs_direct(E, O, gpu, method):
    vmesh, pmesh, ufesp, pfesp = stokes_setup(E, 16, lid=True)
    K0, n = stokes_oracle_K(E, O, vmesh, ufesp, pfesp)
    nu = E.nunknowns(ufesp) + E.nunknowns(pfesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_stokes(am, E.FEIterator(ufesp), E.FEIterator(pfesp), E.QPIterator(ufesp, {"npts": 3}), 1.0)
    U = np.zeros(n)
    E.gathersysvec(U, [ufesp, pfesp])
    U0 = O.solve_lifted(K0, np.zeros(n), U.copy(), nu)
    st = E.solve(U, am, None, nu, method=method, rtol=1e-10, maxit=50000)
    assert st["converged"]
    nv = E.nunknowns(ufesp)
    assert np.abs(U[:nv] - U0[:nv]).max() / np.abs(U0[:nv]).max() < 1e-6
