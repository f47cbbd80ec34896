"""The CPU oracle against the reference's own golden vectors (no GPU).

Each test restates a known-answer test of the Elfel.jl suite; the numbers
come from tests/golden/*.json (extracted from the reference's test files).
"""
import numpy as np
import pytest

from problems import heat_space, stokes_errors, stokes_oracle_K, stokes_setup


def test_quadrature_and_basis(O, golden):
    g = golden("qpiterators.json")
    pc, w = O.quadrature_triangle(3)
    assert np.allclose(pc, g["tri3_param_coords"]) and np.allclose(w, g["tri3_weights"])
    assert all(x == g["weight_3pt"] for x in w)  # test_qpiterators.jl:58-61 asserts equality
    N, G = O.bfun_tables(3, pc)
    assert np.allclose(N, g["t3_3pt_N"])
    for q in range(3):
        assert np.allclose(G[q], g["t3_gradpar"])
    pc1, w1 = O.quadrature_triangle(1)
    N1, _ = O.bfun_tables(3, pc1)
    assert np.allclose(N1, g["t3_1pt_N"])


def test_sparse_7x7_duplicates(O, golden):
    """test/test_assemblers.jl:6-34: COO with duplicates -> dense reference B."""
    g = golden("assemblers.json")
    I, J, V = [], [], []
    for blk in g["blocks"]:
        m = np.array(blk["m"])
        for j in range(m.shape[1]):
            for i in range(m.shape[0]):
                I.append(blk["gi"][i] - 1)
                J.append(blk["gj"][j] - 1)
                V.append(m[i, j])
    A = O.sparse(np.array(I), np.array(J), np.array(V), 7, 7).toarray()
    B = np.array(g["B"])
    assert np.linalg.norm(A - B) / np.linalg.norm(B) < g["rtol"]


def test_sparse_keeps_zeros_and_order(O):
    rng = np.random.default_rng(0)
    I = rng.integers(0, 20, 500)
    J = rng.integers(0, 15, 500)
    V = rng.standard_normal(500)
    V[::7] = 0.0
    K = O.sparse(I, J, V, 20, 15)
    # every distinct (i, j) is a stored entry, zeros included
    assert K.nnz == len(set(zip(I.tolist(), J.tolist())))
    # sums in input order, bit for bit
    ref = {}
    for i, j, v in zip(I, J, V):
        ref[(i, j)] = ref[(i, j)] + v if (i, j) in ref else v
    for j in range(15):
        for k in range(K.indptr[j], K.indptr[j + 1]):
            assert K.data[k] == ref[(K.indices[k], j)]


def test_numbering_qmesh(O, golden):
    """test/test_feiterators.jl:21-71 and :140-172 on the qmesh fixture."""
    gm = golden("meshes.json")
    g = golden("feiterators.json")
    conn = gm["qmesh_conn"]
    assert conn == g["qmesh_conn"]
    f = O.FieldOracle(1, 12)
    for i in g["ebc_nodes"]:
        f.setebc(i, 1, 0.0)
    O.numberdofs([f])
    assert [f.dofnums[n][0] for n in range(12)] == g["scalar_dofnum_by_node"]
    assert f.nunknowns() == g["scalar_nunknowns_ebc"]
    f3 = O.FieldOracle(3, 12)
    for i in g["ebc_nodes"]:
        f3.setebc(i, 1, 0.0)
    O.numberdofs([f3])
    assert O.eldofs(conn, f3) == g["vec3_eldofs"]


def test_element_by_element_dense(O, golden):
    """test/test_feiterators.jl:88-119: sparse assembly equals the dense scatter."""
    gm = golden("meshes.json")
    g = golden("feiterators.json")
    f = O.FieldOracle(1, 12)
    for i in g["ebc_nodes"]:
        f.setebc(i, 1, 0.0)
    O.numberdofs([f])
    ed = np.array(O.eldofs(gm["qmesh_conn"], f)) - 1
    A = np.array(g["A"])
    ke = np.tile(A.ravel(order="F"), (ed.shape[0], 1))
    S = O.sparse(*O.local_coo(ed, ed, ke), 12, 12).toarray()
    D = np.zeros((12, 12))
    for d in ed:
        D[np.ix_(d, d)] += A
    assert np.allclose(S, D)


def test_fefields_mt3gen3(O, golden):
    """test/test_fefields.jl:13-52."""
    gm = golden("meshes.json")
    g = golden("fefields.json")
    nt = len(gm["mt3gen3_xyz"])
    f = O.FieldOracle(2, nt)
    f.numberfreedofs()
    f.numberdatadofs(f.freedofnums()[1] + 1)
    assert f.freedofnums()[1] == g["highest_free_no_ebc"]
    for tid, comp, val in g["ebc"]:
        f.setebc(tid, comp, val)
    f.numberfreedofs(1)
    f.numberdatadofs(f.freedofnums()[1] + 1)
    assert f.freedofnums()[1] == g["highest_free_ebc"]
    assert f.datadofnums()[1] == g["highest_data_ebc"]
    v = O.gathersysvec([0.0] * (nt * 2), f)
    assert v[nt * 2 - 2] == 3.0


def test_heat_t3_golden(E, O, golden):
    """test/test_heat.jl:78-110: T3, N=4, 1-point rule: golden T and exact nodal values."""
    g = golden("heat_t3.json")
    mesh = E.T3block(g["A"], g["A"], g["N"], g["N"])
    fesp = heat_space(E, mesh, E.FEH1_T3())
    elit = E.FEIterator(fesp)
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    # the oracle's own numbering restatement, checked against the host numbering
    f = O.FieldOracle(1, mesh.nnodes)
    for b in E.boundary_nodes(mesh):
        f.setebc(int(b), 1, 0.0)
    O.numberdofs([f])
    assert (np.array(O.eldofs(mesh.conn.tolist(), f)) == elit.eldofs_table()).all()
    K, F = O.assemble_heat(3, 1, mesh.conn - 1, mesh.xy, elit.eldofs_table() - 1, n, g["kappa"], g["Q"])
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    T = O.solve_lifted(K, F, T, nu)
    assert np.allclose(T, g["T"], rtol=1e-8, atol=1e-12)
    ex = 1.0 + mesh.xy[:, 0] ** 2 + 2 * mesh.xy[:, 1] ** 2
    nodal = T[fesp.field.dofnums[:, 0] - 1]
    assert np.mean(np.abs(nodal - ex)) <= g["mean_nodal_error_max"]


def test_stokes_counts(E, golden):
    """test/test_stokes.jl:130: Taylor-Hood DOF counts of the driven cavity at N=100."""
    g = golden("stokes.json")
    N = g["driven_cavity_N"]
    vmesh = E.T6block(1.0, 1.0, N, N)
    pmesh = E.T6toT3(vmesh)
    ux = E.FESpace(float, vmesh, E.FEH1_T6(), 1)
    uy = E.FESpace(float, vmesh, E.FEH1_T6(), 1)
    p = E.FESpace(float, pmesh, E.FEH1_T3(), 1)
    bn = E.boundary_nodes(vmesh)
    E.setebc(ux, 0, bn, 1, 0.0)
    E.setebc(uy, 0, bn, 1, 0.0)
    E.setebc(p, 0, 1, 1, 0.0)
    E.numberdofs([ux, uy, p])
    tndof = E.ndofs(ux) + E.ndofs(uy) + E.ndofs(p)
    tnunk = E.nunknowns(ux) + E.nunknowns(uy) + E.nunknowns(p)
    assert [tndof, tnunk] == g["driven_cavity_tndof_tnunk"]


def test_stokes_veclap_errors(E, O, golden):
    """test/test_stokes.jl:777-780: vector-Laplacian Taylor-Hood, N=4, (ep, ev)."""
    g = golden("stokes.json")["veclap_th_errors"]
    vmesh, pmesh, ufesp, pfesp = stokes_setup(E, g["N"])
    K, n = stokes_oracle_K(E, O, vmesh, ufesp, pfesp)
    U = np.zeros(n)
    E.gathersysvec(U, [ufesp, pfesp])
    nu = E.nunknowns(ufesp) + E.nunknowns(pfesp)
    U = O.solve_lifted(K, np.zeros(n), U, nu)
    ep, ev = stokes_errors(O, vmesh, pmesh, ufesp, pfesp, U)
    assert np.allclose([ep, ev], g["ep_ev"], rtol=1e-8)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_stokes_reddy_errors(E, O, golden, k):
    """test/test_stokes.jl:551-558: Taylor-Hood with scalar velocity spaces, N=4,8,16."""
    g = golden("stokes.json")["reddy_th_errors"]
    N = g["N"][k]
    A = 1.0
    vmesh = E.T6block(2 * A, 2 * A, N, N)
    vmesh = E.Mesh("T6", vmesh.conn, vmesh.xy - A)
    pmesh = E.T6toT3(vmesh)
    ux = E.FESpace(float, vmesh, E.FEH1_T6(), 1)
    uy = E.FESpace(float, vmesh, E.FEH1_T6(), 1)
    ps = E.FESpace(float, pmesh, E.FEH1_T3(), 1)
    fx = lambda x, y: 20 * x * y ** 3
    fy = lambda x, y: 5 * x ** 4 - 5 * y ** 4
    fp = lambda x, y: 60 * x ** 2 * y - 20 * y ** 3
    xy = vmesh.xy
    for box in ([-A, A, -A, -A], [-A, -A, -A, A], [A, A, -A, A], [-A, A, A, A]):
        vl = E.vselect(xy, box, A / N / 100)
        E.setebc(ux, 0, vl, 1, fx(xy[vl - 1, 0], xy[vl - 1, 1]))
        E.setebc(uy, 0, vl, 1, fy(xy[vl - 1, 0], xy[vl - 1, 1]))
    E.setebc(ps, 0, E.vselect_nearest(pmesh.xy, [0.0, 0.0]), 1, 0.0)
    E.numberdofs([ux, uy, ps])
    n = E.ndofs(ux) + E.ndofs(uy) + E.ndofs(ps)
    nu = E.nunknowns(ux) + E.nunknowns(uy) + E.nunknowns(ps)
    dx = E.FEIterator(ux).eldofs_table() - 1
    dy = E.FEIterator(uy).eldofs_table() - 1
    dp = E.FEIterator(ps).eldofs_table() - 1
    kxx, kyy, kxy, kxp, kyp = O.stokes_reddy_element_matrices(3, vmesh.conn - 1, pmesh.conn - 1, vmesh.xy, pmesh.xy,
                                                              1.0)
    parts = [O.local_coo(dx, dx, kxx), O.local_coo(dx, dy, kxy), O.local_coo_transpose(dx, dy, kxy),
             O.local_coo(dy, dy, kyy), O.local_coo(dx, dp, kxp), O.local_coo_transpose(dx, dp, kxp),
             O.local_coo(dy, dp, kyp), O.local_coo_transpose(dy, dp, kyp)]
    ne = vmesh.nel
    I, J, V = (np.concatenate([p[a].reshape(ne, -1) for p in parts], axis=1).ravel() for a in range(3))
    K = O.sparse(I, J, V, n, n)
    U = np.zeros(n)
    E.gathersysvec(U, [ux, uy, ps])
    U = O.solve_lifted(K, np.zeros(n), U, nu)
    pv = U[ps.field.dofnums[:, 0] - 1]
    ep = O.l2_error_scalar(pmesh.conn - 1, pmesh.xy, 3, pv, fp)
    ev = O.l2_error_vector(vmesh.conn - 1, vmesh.xy, 6, U[ux.field.dofnums[:, 0] - 1], U[uy.field.dofnums[:, 0] - 1],
                           fx, fy)
    assert np.allclose([ep, ev], g["ep_ev"][k], rtol=1e-8)
