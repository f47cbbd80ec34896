"""Problem set-ups shared by the tests (mirroring the reference's test drivers)."""
import numpy as np


def tempf(x, y):
    """Exact temperature of test/test_heat.jl:25."""
    return 1.0 + x ** 2 + 2.0 * y ** 2


def heat_space(E, mesh, fe):
    """FESpace with T = tempf on the boundary, numbered (test/test_heat.jl:89-100)."""
    fesp = E.FESpace(float, mesh, fe)
    bn = E.boundary_nodes(mesh)
    E.setebc(fesp, 0, bn, 1, tempf(mesh.xy[bn - 1, 0], mesh.xy[bn - 1, 1]))
    E.numberfreedofs(fesp)
    E.numberdatadofs(fesp)
    return fesp


def heat_oracle(E, O, mesh, fesp, npts, kappa, Q):
    elit = E.FEIterator(fesp)
    n = E.ndofs(fesp)
    return O.assemble_heat(mesh.nodes_per_elem, npts, mesh.conn - 1, mesh.xy, elit.eldofs_table() - 1, n, kappa, Q)


def elasticity_setup(E, nx, ny, Lx=2.0, Ly=1.0, etype="T6", seed=3):
    """Rectangle clamped on the left edge, traction on the right, body force per element."""
    mesh = (E.T6block if etype == "T6" else E.T3block)(Lx, Ly, nx, ny)
    fe = E.FEH1_T6() if etype == "T6" else E.FEH1_T3()
    fesp = E.FESpace(float, mesh, fe, 2)
    left = E.vselect(mesh.xy, [0.0, 0.0, 0.0, Ly], inflate=Lx / nx / 100)
    E.setebc(fesp, 0, left, 1, 0.0)
    E.setebc(fesp, 0, left, 2, 0.0)
    E.numberdofs(fesp)
    rng = np.random.default_rng(seed)
    bforce = rng.uniform(-0.1, 0.1, size=(mesh.nel, 2))
    be = E.boundary_edges(mesh)
    # right-edge boundary edges: both end vertices at x = Lx
    c = mesh.conn - 1
    le = be[:, 1] - 1
    a = c[be[:, 0] - 1, le]
    b = c[be[:, 0] - 1, (le + 1) % 3]
    right = be[(np.abs(mesh.xy[a, 0] - Lx) < 1e-12) & (np.abs(mesh.xy[b, 0] - Lx) < 1e-12)]
    return mesh, fesp, bforce, right


def elasticity_D(Em, nu, plane_strain=True):
    if plane_strain:
        f = Em / ((1 + nu) * (1 - 2 * nu))
        return np.array([[f * (1 - nu), f * nu, 0], [f * nu, f * (1 - nu), 0], [0, 0, f * (1 - 2 * nu) / 2]])
    f = Em / (1 - nu * nu)
    return np.array([[f, f * nu, 0], [f * nu, f, 0], [0, 0, f * (1 - nu) / 2]])


def traction_oracle(mesh, edofs0, edges, t, n):
    """Consistent nodal loads of a constant traction on straight edges:
    [1/2, 1/2] L for T3 edges, [1/6, 1/6, 4/6] L for T6 edges (end, end, midside)."""
    F = np.zeros(n)
    c = mesh.conn - 1
    nn = mesh.nodes_per_elem
    for e, le in edges - 1:
        a, b = c[e, le], c[e, (le + 1) % 3]
        L = np.hypot(*(mesh.xy[b] - mesh.xy[a]))
        nodes = [le, (le + 1) % 3] + ([3 + le] if nn == 6 else [])
        w = [0.5, 0.5] if nn == 3 else [1 / 6, 1 / 6, 4 / 6]
        for ln, wk in zip(nodes, w):
            for comp in range(2):
                F[edofs0[e, 2 * ln + comp]] += wk * L * t[comp]
    return F


def stokes_setup(E, N, A=1.0, lid=False):
    """Taylor-Hood spaces of test/test_stokes.jl:697-753 (colliding flow) or the driven cavity."""
    if lid:
        vmesh = E.T6block(A, A, N, N)
    else:
        vmesh = E.T6block(2 * A, 2 * A, N, N)
        vmesh = E.Mesh("T6", vmesh.conn, vmesh.xy - A)
    pmesh = E.T6toT3(vmesh)
    ufesp = E.FESpace(float, vmesh, E.FEH1_T6(), 2)
    pfesp = E.FESpace(float, pmesh, E.FEH1_T3(), 1)
    infl = A / N / 100
    xy = vmesh.xy
    if lid:
        for box in ([0.0, A, 0.0, 0.0], [0.0, 0.0, 0.0, A], [A, A, 0.0, A]):
            vl = E.vselect(xy, box, infl)
            E.setebc(ufesp, 0, vl, 1, 0.0)
            E.setebc(ufesp, 0, vl, 2, 0.0)
        vl = E.vselect(xy, [0.0, A, A, A], infl)
        E.setebc(ufesp, 0, vl, 1, 1.0)
        E.setebc(ufesp, 0, vl, 2, 0.0)
        E.setebc(pfesp, 0, 1, 1, 0.0)
    else:
        ux = lambda x, y: 20 * x * y ** 3
        uy = lambda x, y: 5 * x ** 4 - 5 * y ** 4
        for box in ([-A, A, -A, -A], [-A, -A, -A, A], [A, A, -A, A], [-A, A, A, A]):
            vl = E.vselect(xy, box, infl)
            E.setebc(ufesp, 0, vl, 1, ux(xy[vl - 1, 0], xy[vl - 1, 1]))
            E.setebc(ufesp, 0, vl, 2, uy(xy[vl - 1, 0], xy[vl - 1, 1]))
        E.setebc(pfesp, 0, E.vselect_nearest(pmesh.xy, [0.0, 0.0]), 1, 0.0)
    E.numberdofs([ufesp, pfesp])
    return vmesh, pmesh, ufesp, pfesp


def stokes_exact():
    return (lambda x, y: 20 * x * y ** 3, lambda x, y: 5 * x ** 4 - 5 * y ** 4,
            lambda x, y: 60 * x ** 2 * y - 20 * y ** 3)


def stokes_oracle_K(E, O, vmesh, ufesp, pfesp, mu=1.0, npts=3):
    """K of test/test_stokes.jl:629-668 by the oracle (kuu, kup, kup')."""
    ud = E.FEIterator(ufesp).eldofs_table() - 1
    pd = E.FEIterator(pfesp).eldofs_table() - 1
    n = E.ndofs(ufesp) + E.ndofs(pfesp)
    kuu, kup = O.stokes_veclap_element_matrices(npts, vmesh.conn - 1, vmesh.xy, mu)
    I1, J1, V1 = O.local_coo(ud, ud, kuu)
    I2, J2, V2 = O.local_coo(ud, pd, kup)
    I3, J3, V3 = O.local_coo_transpose(ud, pd, kup)
    E_ = vmesh.nel
    # append order per element: kuu, kup, transpose(kup)
    I = np.concatenate([I1.reshape(E_, -1), I2.reshape(E_, -1), I3.reshape(E_, -1)], axis=1).ravel()
    J = np.concatenate([J1.reshape(E_, -1), J2.reshape(E_, -1), J3.reshape(E_, -1)], axis=1).ravel()
    V = np.concatenate([V1.reshape(E_, -1), V2.reshape(E_, -1), V3.reshape(E_, -1)], axis=1).ravel()
    return O.sparse(I, J, V, n, n), n


def stokes_errors(O, vmesh, pmesh, ufesp, pfesp, U):
    """(ep, ev) of test/test_stokes.jl:716-760 from the system vector U."""
    ux, uy, p = stokes_exact()
    uf = ufesp.field
    pf = pfesp.field
    uvals = U[uf.dofnums - 1]  # nnodes x 2
    pvals = U[pf.dofnums[:, 0] - 1]
    ep = O.l2_error_scalar(pmesh.conn - 1, pmesh.xy, 3, pvals, p)
    ev = O.l2_error_vector(vmesh.conn - 1, vmesh.xy, 6, uvals[:, 0], uvals[:, 1], ux, uy)
    return ep, ev
