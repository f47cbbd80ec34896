"""Element library beyond T3/T6 (host side and oracle, no GPU).

Pins, against the reference's own tests (tests/golden/elements.json):
  quadrature rules    test/test_refshapes.jl (interval, square, triangle, tetrahedron)
  elements            test/test_felements.jl (L2, T4, FEL2_Q4, FEL2_T4, FEL2_T3)
  bubble space        test/test_fespaces.jl:85-172
  Q4 heat             test/test_heat.jl:120-220 (unknowns at N = 100, nodal error)
  T4 heat             examples/heat/poisson/t4.jl:73-85 (nodal error)
The host iterators (FEIterator/QPIterator/jacjac/bfungrad) are checked
against the oracle's element matrices for Q4, T4 and the bubble element.
"""
import numpy as np
import pytest

from problems import heat_space, tempf

RTOL = 1.4901161193847656e-08  # Julia's isapprox default: sqrt(eps(Float64))


def close(a, b, rtol=RTOL):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def test_quadrature_rules(E, golden):
    g = golden("elements.json")
    qr = E.quadrature(E.RefShapeInterval)
    assert E.npts(qr) == g["interval_default_npts"]
    qr = E.quadrature(E.RefShapeInterval, {"order": 3})
    assert close(E.param_coords(qr).ravel(), g["interval_order3"]["param_coords"])
    assert close(E.weights(qr), g["interval_order3"]["weights"])
    res = []
    for n in range(1, 11):
        qr = E.quadrature(E.RefShapeInterval, {"order": n})
        res.append(np.sum(np.exp(E.param_coords(qr).ravel()) * E.weights(qr)))
    assert close(res, g["interval_exp_integrals"])
    assert E.npts(E.quadrature(E.RefShapeSquare)) == 1
    qr = E.quadrature(E.RefShapeSquare, {"order": 2})
    assert E.npts(qr) == 4 and close(E.param_coords(qr)[2], g["square_order2_point3"])
    lo, hi = g["square_orders"]
    for o in range(lo, hi + 1):
        qr = E.quadrature(E.RefShapeSquare, {"kind": "Gauss", "order": o})
        assert E.npts(qr) == o * o
        assert abs(E.weights(qr).sum() - 4.0) < 1e-12
    for n in g["triangle_npts"]:
        qr = E.quadrature(E.RefShapeTriangle, {"npts": n})
        assert E.npts(qr) == n
        # every rule integrates 1 and x + y exactly, up to its tabulated decimals
        assert abs(E.weights(qr).sum() - 0.5) < 1e-12
        assert abs(E.weights(qr) @ E.param_coords(qr).sum(axis=1) - 1.0 / 3.0) < 1e-8
    for t in g["tetrahedron"]:
        qr = E.quadrature(E.RefShapeTetrahedron, {"npts": t["npts"]})
        assert E.npts(qr) == t["npts"]
        assert close(E.param_coords(qr), t["param_coords"])
        assert close(E.weights(qr), t["weights"])
    with pytest.raises(ValueError):
        E.quadrature(E.RefShapeTriangle, {"npts": 5})
    with pytest.raises(ValueError):
        E.quadrature(E.RefShapeSquare, {"kind": "Lobatto"})


def test_elements(E, golden):
    g = golden("elements.json")
    fe = E.FEH1_L2()
    assert E.refshape(fe) is E.RefShapeInterval and E.manifdim(fe) == 1
    assert [E.ndofperfeat(fe, m) for m in range(4)] == [1, 0, 0, 0]
    assert close(fe.bfun([1 / 3]), g["L2"]["bfun_at_one_third"])
    assert close(fe.bfungradpar([1 / 3]), g["L2"]["gradpar"])
    fe = E.FEH1_T4()
    assert close(fe.bfungradpar([0.25] * 3), g["T4_gradpar"])
    for name, c in g["counts"].items():
        fe = getattr(E, name)()
        assert [E.nfeatofdim(fe, m) for m in range(4)] == c["nfeatofdim"], name
        assert [E.ndofperfeat(fe, m) for m in range(4)] == c["ndofperfeat"], name
        pc = [0.25] * E.manifdim(fe)
        assert close(fe.bfun(pc), c["bfun"]), name
        assert np.all(fe.bfungradpar(pc) == 0.0) or name == "FEH1_T4"
    # Q4: partition of unity, gradients sum to zero, nodal interpolation
    fe = E.FEH1_Q4()
    corners = [[-1, -1], [1, -1], [1, 1], [-1, 1]]
    for k, pc in enumerate(corners):
        assert np.allclose(fe.bfun(pc), np.eye(4)[k])
    rng = np.random.default_rng(1)
    for pc in rng.uniform(-1, 1, (5, 2)):
        assert abs(fe.bfun(pc).sum() - 1) < 1e-15 and np.abs(fe.bfungradpar(pc).sum(axis=0)).max() < 1e-15
    assert E.FEL2_Q4().geometrycarrier() == E.FEH1_Q4()
    assert E.FEL2_T4().geometrycarrier() == E.FEH1_T4()
    assert E.FEH1_T3_BUBBLE().geometrycarrier() == E.FEH1_T3_BUBBLE()


def test_jacobians(E):
    J3 = np.array([[2.0, 0.1, 0.0], [0.0, 3.0, 0.2], [0.1, 0.0, 4.0]])
    assert abs(E.Jacobian(J3) - np.linalg.det(J3)) < 1e-12
    assert abs(E.Jacobian(np.array([[3.0], [4.0]])) - 5.0) < 1e-15  # curve in the plane
    J32 = np.array([[1.0, 0.0], [0.0, 2.0], [0.0, 0.0]])  # surface in space
    assert abs(E.Jacobian(J32) - 2.0) < 1e-15


def test_bubble_space(E, golden):
    """test/test_fespaces.jl:85-172 on a T3 block mesh (the qmesh fixture is a T3 mesh too)."""
    g = golden("elements.json")["bubble"]
    mesh = E.T3block(1.0, 1.0, 3, 2)
    for ncomp in (1, 2):
        fesp = E.FESpace(float, mesh, E.FEH1_T3_BUBBLE(), ncomp)
        fe = fesp.fe
        assert [E.nfeatofdim(fe, m) for m in range(4)] == g["nfeatofdim"]
        assert [E.ndofperfeat(fe, m) for m in range(4)] == g["ndofperfeat"]
        assert E.fe_ndofsperel(fe) == g["ndofsperel"]
        assert close(fe.bfun([1 / 3, 1 / 3]), g["bfun_at_one_third"])
        # the reference test's own loop for the element DOF layout
        emdim, bfnum, compnt, bfn = [], [], [], 1
        for m in range(4):
            if E.ndofperfeat(fe, m) > 0:
                for _ in range(E.nfeatofdim(fe, m)):
                    for _k in range(E.ndofperfeat(fe, m)):
                        for j in range(1, ncomp + 1):
                            emdim.append(m)
                            bfnum.append(bfn)
                            compnt.append(j)
                        bfn += 1
        assert list(E.edofmdim(fesp)) == emdim
        assert list(E.edofbfnum(fesp)) == bfnum
        assert list(E.edofcompnt(fesp)) == compnt
        assert E.dofnum(fesp, 0, 1, 1) == 0
        # numbered: node DOFs, then cell DOFs; the iterator lists them in that order
        E.setebc(fesp, 0, E.boundary_nodes(mesh), 1, 0.0)
        E.numberdofs(fesp)
        nnodes, nel = mesh.nnodes, mesh.nel
        assert E.ndofs(fesp) == (nnodes + nel) * ncomp
        nb = len(E.boundary_nodes(mesh))
        assert E.nunknowns(fesp) == (nnodes + nel) * ncomp - nb
        elit = E.FEIterator(fesp)
        tab = elit.eldofs_table()
        assert tab.shape == (nel, 4 * ncomp)
        for el in elit:
            e = el._state
            d = E.eldofs(el)
            assert list(d) == list(tab[e - 1])
            assert list(d[3 * ncomp:]) == [E.dofnum(fesp, 2, e, c) for c in range(1, ncomp + 1)]
            assert list(E.eldofentmdims(el)) == [0] * (3 * ncomp) + [2] * ncomp
            assert list(E.eldofcomps(el)) == list(range(1, ncomp + 1)) * 4
            if e == 3:
                break
        # every number 1..ndofs is used once
        allnums = np.concatenate([f.dofnums.ravel() for f in fesp._fields.values()])
        assert np.array_equal(np.sort(allnums), np.arange(1, E.ndofs(fesp) + 1))


def test_cell_constant_space(E):
    """FEL2_Q4 (pressure of the Q1-Q0 Stokes examples): one DOF per cell,
    geometry from FEH1_Q4."""
    mesh = E.Q4block(2.0, 1.0, 4, 3)
    fesp = E.FESpace(float, mesh, E.FEL2_Q4(), 1)
    E.setebc(fesp, 2, 1, 1, 0.0)
    E.numberdofs(fesp)
    assert E.ndofs(fesp) == mesh.nel and E.nunknowns(fesp) == mesh.nel - 1
    elit = E.FEIterator(fesp)
    qpit = E.QPIterator(fesp, {"kind": "Gauss", "order": 2})
    area = 0.0
    for el in elit:
        for qp in qpit:
            _, J = E.jacjac(el, qp)
            area += J * E.weight(qp)
            assert E.bfun(qp).tolist() == [1.0]
    assert abs(area - 2.0) < 1e-12


def _iter_heat(E, fesp, qargs, kappa, Q, count):
    """ke, fe of the first `count` elements by the reference's integrate! loop
    (test/test_heat.jl:151-171) over the host iterators."""
    elit = E.FEIterator(fesp)
    qpit = E.QPIterator(fesp, qargs)
    n = E.ndofsperel(fesp)
    out = []
    for el in elit:
        ke = np.zeros((n, n))
        fe = np.zeros(n)
        for qp in qpit:
            Jac, J = E.jacjac(el, qp)
            gradN = E.bfungrad(qp, Jac)
            JxW = J * E.weight(qp)
            N = E.bfun(qp)
            ke += gradN @ gradN.T * (kappa * JxW)
            fe += N * Q * JxW
        out.append((ke, fe))
        if len(out) == count:
            break
    return out


@pytest.mark.parametrize("kind", ["Q4", "T4", "T3B"])
def test_host_iterators_vs_oracle(E, O, kind):
    if kind == "Q4":
        mesh = E.jitter(E.Q4block(1.0, 1.0, 4, 4), 0.05, seed=3)
        fe, qargs = E.FEH1_Q4(), {"kind": "Gauss", "order": 2}
        pc, w = O.quadrature_square(2)
        ng = None
    elif kind == "T4":
        mesh = E.jitter(E.T4block(1.0, 1.0, 1.0, 2, 2, 2), 0.05, seed=3)
        fe, qargs = E.FEH1_T4(), {"npts": 4}
        pc, w = O.quadrature_tetrahedron(4)
        ng = None
    else:
        mesh = E.jitter(E.T3block(1.0, 1.0, 3, 3), 0.05, seed=3)
        fe, qargs = E.FEH1_T3_BUBBLE(), {"npts": 3}
        pc, w = O.quadrature_triangle(3)
        ng = 3
    fesp = E.FESpace(float, mesh, fe)
    E.numberdofs(fesp)
    got = _iter_heat(E, fesp, qargs, 1.5, -2.0, 6)
    conn = mesh.conn - 1
    if kind == "T3B":
        conn = np.concatenate([conn, conn[:, :1]], axis=1)  # 4 basis functions, 3 geometry nodes
    ke, fe0 = O.heat_element_matrices_iso(kind, pc, w, conn[:6], mesh.xy, 1.5, -2.0, nodes_geom=ng)
    nb = int(round(np.sqrt(ke.shape[1])))
    for e, (k, f) in enumerate(got):
        assert np.abs(k - ke[e].reshape(nb, nb).T).max() <= 1e-13 * np.abs(k).max()
        assert np.abs(f - fe0[e]).max() <= 1e-13 * np.abs(f).max()


def test_q4_heat_known_answer(E, O, golden):
    """test/test_heat.jl:120-220 through the oracle: N = 100 Q4 block, 2 x 2
    Gauss, 9801 unknowns, mean nodal error of the solution <= 1e-9."""
    g = golden("elements.json")["heat_q4"]
    mesh = E.Q4block(1.0, 1.0, g["N"], g["N"])
    fesp = heat_space(E, mesh, E.FEH1_Q4())
    assert E.nunknowns(fesp) == g["nunknowns"]
    pc, w = O.quadrature_square(g["order"])
    ke, fe = O.heat_element_matrices_iso("Q4", pc, w, mesh.conn - 1, mesh.xy, g["kappa"], g["Q"])
    ed = E.FEIterator(fesp).eldofs_table() - 1
    n = E.ndofs(fesp)
    K = O.sparse(*O.local_coo(ed, ed, ke), n, n)
    F = O.vec_assemble(n, ed, fe)
    T = E.gathersysvec(np.zeros(n), fesp)
    T = O.solve_lifted(K, F, T, E.nunknowns(fesp))
    E.scattersysvec(fesp, T)
    err = np.abs(fesp.field.dofvals[:, 0] - tempf(mesh.xy[:, 0], mesh.xy[:, 1])).mean()
    assert err <= g["mean_nodal_error_max"]


def test_t4_heat_known_answer(E, O):
    """examples/heat/poisson/t4.jl:73-85 through the oracle on a smaller
    cube (N = 8 instead of 20): mean nodal error <= 1e-9."""
    N = 8
    mesh = E.T4block(1.0, 1.0, 1.0, N, N, N)
    fesp = heat_space(E, mesh, E.FEH1_T4())
    assert E.nunknowns(fesp) == (N - 1) ** 3
    pc, w = O.quadrature_tetrahedron(1)
    ke, fe = O.heat_element_matrices_iso("T4", pc, w, mesh.conn - 1, mesh.xy, 1.0, -6.0)
    ed = E.FEIterator(fesp).eldofs_table() - 1
    n = E.ndofs(fesp)
    K = O.sparse(*O.local_coo(ed, ed, ke), n, n)
    F = O.vec_assemble(n, ed, fe)
    T = O.solve_lifted(K, F, E.gathersysvec(np.zeros(n), fesp), E.nunknowns(fesp))
    E.scattersysvec(fesp, T)
    err = np.abs(fesp.field.dofvals[:, 0] - tempf(mesh.xy[:, 0], mesh.xy[:, 1])).mean()
    assert err <= 1e-9


def test_meshes(E):
    q = E.Q4block(2.0, 1.0, 3, 2)
    assert q.conn.shape == (6, 4) and q.nnodes == 12
    X = q.xy[q.conn - 1]
    d1, d2 = X[:, 2] - X[:, 0], X[:, 3] - X[:, 1]
    area = 0.5 * np.abs(d1[:, 0] * d2[:, 1] - d1[:, 1] * d2[:, 0])
    assert abs(area.sum() - 2.0) < 1e-14
    assert len(E.boundary_nodes(q)) == 10
    t = E.T4block(1.0, 2.0, 3.0, 2, 3, 4)
    assert t.conn.shape == (6 * 24, 4) and t.sdim == 3
    X = t.xy[t.conn - 1]
    det = np.linalg.det(np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], axis=2))
    assert det.min() > 0 and abs(det.sum() / 6 - 6.0) < 1e-12
    assert len(E.boundary_nodes(t)) == t.nnodes - 1 * 2 * 3
    s = E.L2block(2.0, 5)
    assert s.conn.tolist()[0] == [1, 2] and E.boundary_nodes(s).tolist() == [1, 6]
    assert E.vselect(t.xy, [0, 0, 0, 2, 0, 3], inflate=1e-9).size == 4 * 5
