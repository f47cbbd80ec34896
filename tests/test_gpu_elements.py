"""Device assembly of the wider element library against the oracle (GPU).

Fused Q4 and T4 heat (heat_q4_k, heat_t4_k): pattern bit-exact, values within
1e-12 of the largest entry; the reference's known answers (test/test_heat.jl:
120-220 for Q4, examples/heat/poisson/t4.jl:73-85 for T4) through the device
assembly and the device solver.  Elements without a fused kernel (the T3 with
a bubble of test/test_stokes.jl:160-285) go through COO mode: the device CSC
is bit-identical to the oracle's sparse() of the same triplets.
"""
import numpy as np
import pytest

from problems import heat_space, tempf

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # FP64 parity tolerance, relative to max |entry|


def same_pattern(K, K0):
    K.sort_indices()
    return (K.indptr == K0.indptr).all() and (K.indices == K0.indices).all() and K.shape == K0.shape


def close(a, b, rtol=RTOL):
    return np.abs(a - b).max() <= rtol * max(np.abs(b).max(), 1e-300)


def _mesh(E, kind, n, jit):
    if kind == "Q4":
        m = E.Q4block(1.0, 1.0, n, n)
    else:
        m = E.T4block(1.0, 1.0, 1.0, n, n, n)
    return E.jitter(m, jit / n, seed=7) if jit else m


def _oracle(E, O, kind, mesh, fesp, rule, kappa, Q):
    if kind == "Q4":
        pc, w = O.quadrature_square(rule)
    else:
        pc, w = O.quadrature_tetrahedron(rule)
    ke, fe = O.heat_element_matrices_iso(kind, pc, w, mesh.conn - 1, mesh.xy, kappa, Q)
    ed = E.FEIterator(fesp).eldofs_table() - 1
    n = E.ndofs(fesp)
    return O.sparse(*O.local_coo(ed, ed, ke), n, n), O.vec_assemble(n, ed, fe)


@pytest.mark.parametrize("kind,n,jit,rule", [("Q4", 5, 0.0, 2), ("Q4", 23, 0.2, 2), ("Q4", 17, 0.15, 3),
                                             ("T4", 3, 0.0, 1), ("T4", 7, 0.15, 4), ("T4", 6, 0.1, 5)])
def test_fused_heat_parity(E, O, gpu, kind, n, jit, rule):
    mesh = _mesh(E, kind, n, jit)
    fesp = heat_space(E, mesh, E.FEH1_Q4() if kind == "Q4" else E.FEH1_T4())
    rng = np.random.default_rng(n)
    kappa = np.exp(rng.uniform(np.log(0.5), np.log(2.0), mesh.nel))
    qs = {"kind": "Gauss", "order": rule} if kind == "Q4" else {"npts": rule}
    N = E.ndofs(fesp)
    am = E.start(E.SysmatAssemblerGPU(), N, N)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, qs), kappa, -6.0)
    K, F = E.finish(am), am.rhs()
    K0, F0 = _oracle(E, O, kind, mesh, fesp, rule, kappa, -6.0)
    assert same_pattern(K, K0)
    assert close(K.data, K0.data) and close(F, F0)
    # coefficients change, pattern reused
    am.heat(kappa * 3.0, 2.0)
    K2, F2 = E.finish(am), am.rhs()
    assert same_pattern(K2, K0) and close(K2.data, 3.0 * K0.data) and close(F2, -F0 / 3.0)
    # tables round-trip with the space's coordinate dimension
    conn, xy, dofs = am.tables()
    assert (conn == mesh.conn).all() and (xy == mesh.xy).all()


def _nodal_error(E, fesp, mesh, T):
    E.scattersysvec(fesp, T)
    return np.abs(fesp.field.dofvals[:, 0] - tempf(mesh.xy[:, 0], mesh.xy[:, 1])).mean()


@pytest.mark.parametrize("kind", ["Q4", "T4"])
def test_known_answer_on_device(E, O, gpu, golden, kind):
    """Q4: N = 100, 2 x 2 Gauss, 9801 unknowns (test/test_heat.jl:207); T4:
    N = 10 cube, one-point rule.  Mean nodal error <= 1e-9 with the device K
    and F solved by the oracle's direct solver, and with the device FP64 PCG."""
    if kind == "Q4":
        g = golden("elements.json")["heat_q4"]
        mesh, fe, qs = E.Q4block(1.0, 1.0, g["N"], g["N"]), E.FEH1_Q4(), {"kind": "Gauss", "order": g["order"]}
    else:
        g = {"kappa": 1.0, "Q": -6.0, "mean_nodal_error_max": 1e-9, "nunknowns": 9 ** 3}
        mesh, fe, qs = E.T4block(1.0, 1.0, 1.0, 10, 10, 10), E.FEH1_T4(), {"npts": 1}
    fesp = heat_space(E, mesh, fe)
    nu = E.nunknowns(fesp)
    assert nu == g["nunknowns"]
    n = E.ndofs(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, qs), g["kappa"], g["Q"])
    K, F = E.finish(am), am.rhs()
    T0 = E.gathersysvec(np.zeros(n), fesp)
    T = O.solve_lifted(K, F, T0, nu)
    assert _nodal_error(E, fesp, mesh, T) <= g["mean_nodal_error_max"]
    T = T0.copy()
    st = E.solve(T, am, None, nu, method="pcg64", rtol=1e-13)
    assert st["converged"]
    assert _nodal_error(E, fesp, mesh, T) <= g["mean_nodal_error_max"]


def test_unsupported_fused_elements(E, gpu):
    mesh = E.T3block(1.0, 1.0, 2, 2)
    fesp = E.FESpace(float, mesh, E.FEH1_T3_BUBBLE())
    E.numberdofs(fesp)
    n = E.ndofs(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    with pytest.raises(E.ElfelError):
        E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.0, 1.0)
    q = E.Q4block(1.0, 1.0, 2, 2)
    fq = E.FESpace(float, q, E.FEH1_Q4(), 2)
    E.numberdofs(fq)
    n = E.ndofs(fq)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    with pytest.raises(E.ElfelError):  # Q4 takes the heat weak form only
        E.assemble_elasticity(am, E.FEIterator(fq), E.QPIterator(fq, {"kind": "Gauss", "order": 2}), 1.0, 0.3)


def test_p1b_p1_stokes_coo(E, O, gpu):
    """The driven-cavity P1b-P1 Stokes assembly of test/test_stokes.jl:160-285
    (bubble-enriched velocity, T3 pressure, mu = 0.25) through COO mode on a
    12 x 12 mesh; the device CSC equals the oracle's sparse() bit for bit."""
    N, A, mu = 12, 1.0, 0.25
    mesh = E.T3block(A, A, N, N)
    ux = E.FESpace(float, mesh, E.FEH1_T3_BUBBLE(), 1)
    uy = E.FESpace(float, mesh, E.FEH1_T3_BUBBLE(), 1)
    inflate = A / N / 100
    for box in ([0.0, A, 0.0, 0.0], [0.0, 0.0, 0.0, A], [A, A, 0.0, A]):
        vl = E.vselect(mesh.xy, box, inflate=inflate)
        E.setebc(ux, 0, vl, 1, 0.0)
        E.setebc(uy, 0, vl, 1, 0.0)
    vl = E.vselect(mesh.xy, [0.0, A, A, A], inflate=inflate)
    E.setebc(ux, 0, vl, 1, 1.0)
    E.setebc(uy, 0, vl, 1, 0.0)
    p = E.FESpace(float, mesh, E.FEH1_T3(), 1)
    E.setebc(p, 0, 1, 1, 0.0)
    E.numberdofs([ux, uy, p])
    tndof = E.ndofs(ux) + E.ndofs(uy) + E.ndofs(p)
    elits = [E.FEIterator(s) for s in (ux, uy, p)]
    qpits = [E.QPIterator(s, {"kind": "default", "npts": 3}) for s in (ux, uy, p)]
    nu_, nv_, np_ = (E.ndofsperel(s) for s in (ux, uy, p))
    kxx = E.LocalMatrixAssembler(nu_, nu_, 0.0)
    kyy = E.LocalMatrixAssembler(nv_, nv_, 0.0)
    kxy = E.LocalMatrixAssembler(nu_, nv_, 0.0)
    kxp = E.LocalMatrixAssembler(nu_, np_, 0.0)
    kyp = E.LocalMatrixAssembler(nv_, np_, 0.0)
    ass = E.start(E.SysmatAssemblerSparse(0.0), tndof, tndof)
    for uxel, uyel, pel in zip(*elits):
        E.init(kxx, E.eldofs(uxel), E.eldofs(uxel))
        E.init(kyy, E.eldofs(uyel), E.eldofs(uyel))
        E.init(kxy, E.eldofs(uxel), E.eldofs(uyel))
        E.init(kxp, E.eldofs(uxel), E.eldofs(pel))
        E.init(kyp, E.eldofs(uyel), E.eldofs(pel))
        for uxqp, uyqp, pqp in zip(*qpits):
            Jac, J = E.jacjac(pel, pqp)
            JxW = J * E.weight(pqp)
            gx = E.bfungrad(uxqp, Jac)
            gy = E.bfungrad(uyqp, Jac)
            Np = E.bfun(pqp)
            kxx.M[:, :] += (mu * JxW) * (2 * np.outer(gx[:, 0], gx[:, 0]) + np.outer(gx[:, 1], gx[:, 1]))
            kyy.M[:, :] += (mu * JxW) * (np.outer(gy[:, 0], gy[:, 0]) + 2 * np.outer(gy[:, 1], gy[:, 1]))
            kxy.M[:, :] += (mu * JxW) * np.outer(gx[:, 0], gy[:, 1])
            kxp.M[:, :] += (-JxW) * np.outer(gx[:, 0], Np)
            kyp.M[:, :] += (-JxW) * np.outer(gy[:, 1], Np)
        for la in (kxx, kxy, E.transpose(kxy), kyy, kxp, E.transpose(kxp), kyp, E.transpose(kyp)):
            E.assemble(ass, la)
    K = E.finish(ass)
    I, J, V = ass.triplets()
    K0 = O.sparse(I - 1, J - 1, V, tndof, tndof)
    assert same_pattern(K, K0) and (K.data == K0.data).all()
    assert abs(K - K.T).max() <= 1e-14 * abs(K).max()  # the saddle-point matrix is symmetric
    U = E.gathersysvec(np.zeros(tndof), [ux, uy, p])
    tnunk = E.nunknowns(ux) + E.nunknowns(uy) + E.nunknowns(p)
    U = O.solve_lifted(K0, np.zeros(tndof), U, tnunk)
    assert np.isfinite(U).all()
    E.scattersysvec([ux, uy, p], U)
    # the bubble DOFs are free and carry the interior enrichment; the lid keeps its value
    assert (ux._fields[2].dofnums > 0).all() and (ux._fields[0].dofvals[vl - 1, 0] == 1.0).all()
