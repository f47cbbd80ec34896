"""CPU oracle for the Elfel.jl assembly + solve path (TEST INFRASTRUCTURE).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It is the checker, never the product: the
GPU library does not depend on it.

Restated from the reference (Elfel.jl v0.4.0), file:line in that project:
  quadrature_triangle     src/RefShapes.jl:113-230, 301-323
  bfun/bfungradpar T3/T6  src/FElements.jl:239-288   (C, elfel_oracle.c)
  FEField numbering       src/FEFields.jl:137-177     (pure-Python loops)
  numberdofs!(spaces)     src/FESpaces.jl:141-173, 250-259
  FEIterator eldofs       src/FEIterators.jl:161-194
  LocalMatrixAssembler    src/LocalAssemblers.jl:68-83 (column-major rows/cols)
  SysmatAssemblerSparse   src/Assemblers.jl:97-123 -> SparseArrays.sparse (C)
  SysvecAssembler         src/Assemblers.jl:215-221
  solve!                  test/test_heat.jl:73-76 (scipy SuperLU stands in
                          for SuiteSparse's factorisation behind ``\\``)
  error norms             test/test_stokes.jl:438-496, 716-760
  Gauss / tetrahedron     src/RefShapes.jl:85-112, 248-281, 325-361
  Q4, T4, T3 bubble, L2   src/FElements.jl:290-470 (numpy; the heat weak
                          form of test/test_heat.jl:151-171 and
                          examples/heat/poisson/t4.jl:32-52 over them)

Parity is pinned by the golden vectors in tests/golden (extracted from the
reference's own tests by tests/golden/make_golden.py).
"""
import ctypes
import os
import subprocess

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_d = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.POINTER(ctypes.c_int64)


def build():
    """Compile elfel_oracle.c into oracle/_build/liboracle.so (gcc, OpenMP)."""
    subprocess.check_call(["make", "-s", "-C", _HERE])
    return os.path.join(_HERE, "_build", "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        src = os.path.join(_HERE, "elfel_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(path)
        L.oracle_sparse.restype = ctypes.c_int64
        L.oracle_pcg.restype = ctypes.c_int
        L.oracle_num_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _p(a, t=_d):
    return a.ctypes.data_as(t)


# ---------------------------------------------------------------- quadrature
def quadrature_triangle(npts=1):
    """Triangle rules of src/RefShapes.jl:113-160 (npts = 1, 3, 4, 6, 7)."""
    if npts == 1:
        pc = [[1.0 / 3.0, 1.0 / 3.0]]
        w = [1.0 / 2.0]
    elif npts == 3:
        pc = [[2.0 / 3, 1.0 / 6], [1.0 / 6, 2.0 / 3], [1.0 / 6, 1.0 / 6]]
        w = [x / 2 for x in (1.0 / 3, 1.0 / 3, 1.0 / 3)]
    elif npts == 4:
        pc = [[0.333333333333333, 0.333333333333333], [0.2, 0.2], [0.6, 0.2], [0.2, 0.6]]
        w = [-0.281250000000000, 0.260416666666667, 0.260416666666667, 0.260416666666667]
    elif npts == 6:
        a, b = 0.816847572980459, 0.091576213509771
        c, d = 0.108103018168070, 0.445948490915965
        pc = [[a, b], [b, a], [b, b], [c, d], [d, c], [d, d]]
        w = [x / 2 for x in [0.109951743655322] * 3 + [0.223381589678011] * 3]
    elif npts == 7:
        a, b = 0.101286507323456, 0.797426958353087
        c, d = 0.470142064105115, 0.059715871789770
        pc = [[a, a], [b, a], [a, b], [c, c], [d, c], [c, d], [0.333333333333333, 0.333333333333333]]
        w = [0.062969590272414] * 3 + [0.066197076394253] * 3 + [0.1125]
    else:
        raise ValueError(f"Unknown number of integration points {npts}")
    return np.array(pc, dtype=np.float64), np.array(w, dtype=np.float64)


def gauss_1d(order):
    """Gauss rule on [-1, 1] (src/RefShapes.jl:85-112): the reference's
    tabulated decimals up to order 5, Golub-Welsch above."""
    tab = {1: ([0.0], [2.0]),
           2: ([-0.577350269189626, 0.577350269189626], [1.0, 1.0]),
           3: ([-0.774596669241483, 0.0, 0.774596669241483], [0.5555555555555556, 0.8888888888888889,
                                                              0.5555555555555556]),
           4: ([-0.86113631159405, -0.33998104358486, 0.33998104358486, 0.86113631159405],
               [0.34785484513745, 0.65214515486255, 0.65214515486255, 0.34785484513745]),
           5: ([-0.906179845938664, -0.538469310105683, 0.0, 0.538469310105683, 0.906179845938664],
               [0.236926885056189, 0.478628670499367, 0.568888888888889, 0.478628670499367, 0.236926885056189])}
    if order in tab:
        x, w = tab[order]
        return np.array(x), np.array(w)
    k = np.arange(1, order, dtype=np.float64)
    b = k / np.sqrt(4 * k * k - 1)
    lam, V = np.linalg.eigh(np.diag(b, 1) + np.diag(b, -1))
    return lam, 2 * V[0] ** 2


def quadrature_square(order=1):
    """Tensor-product Gauss rule, first coordinate outer (src/RefShapes.jl:325-361)."""
    x, w = gauss_1d(order)
    pc = np.array([[x[i], x[j]] for i in range(order) for j in range(order)])
    return pc, np.array([w[i] * w[j] for i in range(order) for j in range(order)])


def quadrature_tetrahedron(npts=1):
    """src/RefShapes.jl:248-281 (npts = 1, 4, 5)."""
    if npts == 1:
        return np.array([[0.25, 0.25, 0.25]]), np.array([1.0 / 6.0])
    if npts == 4:
        a, b = 0.13819660, 0.58541020
        return np.array([[a, a, a], [b, a, a], [a, b, a], [a, a, b]]), np.full(4, 1.0 / 24.0)
    if npts == 5:
        a = 1.0 / 6.0
        pc = [[0.25, 0.25, 0.25], [0.5, a, a], [a, 0.5, a], [a, a, 0.5], [a, a, a]]
        return np.array(pc), np.array([-0.8, 0.45, 0.45, 0.45, 0.45]) / 6
    raise ValueError(f"Unknown number of integration points {npts}")


def basis(kind, pc):
    """(N, gradNpar) of one scalar element at one parametric point
    (src/FElements.jl:199-470): kind in Q4, T4, T3B (T3 with bubble), L2."""
    if kind == "Q4":
        x, y = pc
        N = 0.25 * np.array([(1 - x) * (1 - y), (1 + x) * (1 - y), (1 + x) * (1 + y), (1 - x) * (1 + y)])
        G = 0.25 * np.array([[-(1 - y), -(1 - x)], [1 - y, -(1 + x)], [1 + y, 1 + x], [-(1 + y), 1 - x]])
        return N, G
    if kind == "T4":
        r, s, t = pc
        return np.array([1 - r - s - t, r, s, t]), np.array([[-1.0, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    if kind == "T3B":
        r, s = pc
        N = np.array([1 - r - s, r, s, (1 - r - s) * r * s])
        G = np.array([[-1.0, -1], [1, 0], [0, 1], [-r * s + (1 - r - s) * s, -r * s + (1 - r - s) * r]])
        return N, G
    if kind == "L2":
        x = pc[0]
        return np.array([(1 - x) / 2, (1 + x) / 2]), np.array([[-0.5], [0.5]])
    raise ValueError(kind)


def heat_element_matrices_iso(kind, pc, w, conn0, X, kappa, Q, nodes_geom=None):
    """Heat element matrices (test/test_heat.jl:151-171) of an isoparametric
    element over all elements at once, one quadrature point at a time:
    J = X^T gradNpar (geometry from the first nodes_geom basis functions),
    gradN = gradNpar J^-1, ke += gradN gradN^T kappa J w, fe += N Q J w."""
    E, nn = conn0.shape
    ng = nn if nodes_geom is None else nodes_geom
    kappa = np.broadcast_to(np.asarray(kappa, dtype=np.float64), (E,))
    Xe = X[conn0[:, :ng]]  # E x ng x sdim
    nb = basis(kind, pc[0])[0].size
    ke = np.zeros((E, nb, nb))
    fe = np.zeros((E, nb))
    for q in range(pc.shape[0]):
        N, G = basis(kind, pc[q])
        J = np.einsum("eka,kb->eab", Xe, G[:ng])  # E x sdim x mdim
        det = np.linalg.det(J)
        g = np.einsum("ib,eba->eia", G, np.linalg.inv(J))  # gradN = G J^-1
        JxW = det * w[q]
        ke += np.einsum("eia,eja->eij", g, g) * (kappa * JxW)[:, None, None]
        fe += N[None, :] * (Q * JxW)[:, None]
    return ke.transpose(0, 2, 1).reshape(E, nb * nb), fe  # column-major per element, as local_coo wants


def bfun_tables(nn, pc):
    """N (npts x nn) and gradNpar (npts x nn x 2) at the points (C restatement)."""
    npts = pc.shape[0]
    N = np.zeros((npts, nn))
    G = np.zeros((npts, nn, 2))
    pc = np.ascontiguousarray(pc, dtype=np.float64)
    rc = lib().oracle_bfun_tables(nn, npts, _p(pc), _p(N), _p(G))
    assert rc == 0
    return N, G


# ---------------------------------------------------------------- numbering
class FieldOracle:
    """Restatement of FEField (src/FEFields.jl:14-281) with plain loops."""

    def __init__(self, ncomp, nterms):
        self.ncomp = ncomp
        self.dofnums = [[0] * ncomp for _ in range(nterms)]
        self.isdatum = [[False] * ncomp for _ in range(nterms)]
        self.dofvals = [[0.0] * ncomp for _ in range(nterms)]

    def setebc(self, tid, comp, val):  # 1-based tid/comp, FEFields.jl:124-128
        self.isdatum[tid - 1][comp - 1] = True
        self.dofvals[tid - 1][comp - 1] = val

    def numberfreedofs(self, firstnum=1):  # FEFields.jl:137-154
        lnum = firstnum
        for n, d in zip(self.dofnums, self.isdatum):
            for j in range(self.ncomp):
                if not d[j]:
                    n[j] = lnum
                    lnum += 1
                else:
                    n[j] = 0

    def numberdatadofs(self, firstnum=1):  # FEFields.jl:164-177
        num = firstnum
        for n, d in zip(self.dofnums, self.isdatum):
            for j in range(self.ncomp):
                if d[j]:
                    n[j] = num
                    num += 1

    def freedofnums(self):  # FEFields.jl:187-201
        t = l = 0
        f = None
        for n, d in zip(self.dofnums, self.isdatum):
            for j in range(self.ncomp):
                if not d[j]:
                    t += 1
                    l = max(l, n[j])
                    f = n[j] if f is None else min(f, n[j])
        return f, l, t

    def datadofnums(self):  # FEFields.jl:219-233
        t = l = 0
        f = None
        for n, d in zip(self.dofnums, self.isdatum):
            for j in range(self.ncomp):
                if d[j]:
                    t += 1
                    l = max(l, n[j])
                    f = n[j] if f is None else min(f, n[j])
        return f, l, t

    def ndofs(self):
        return len(self.dofnums) * self.ncomp

    def nunknowns(self):
        return self.freedofnums()[2]


def numberdofs(fields):
    """numberdofs!(::AbstractVector) of src/FESpaces.jl:250-259."""
    fields[0].numberfreedofs(1)
    for i in range(1, len(fields)):
        fields[i].numberfreedofs(fields[i - 1].freedofnums()[1] + 1)
    fields[0].numberdatadofs(fields[-1].freedofnums()[1] + 1)
    for i in range(1, len(fields)):
        fields[i].numberdatadofs(fields[i - 1].datadofnums()[1] + 1)


def eldofs(conn1, field):
    """Element DOF table, node-major component-minor (FEIterators.jl:161-171).

    conn1: element node lists, 1-based.  Returns a list of lists (1-based DOFs).
    """
    out = []
    for c in conn1:
        d = []
        for n in c:
            d.extend(field.dofnums[n - 1])
        out.append(d)
    return out


def gathersysvec(v, field):  # FEFields.jl:247-257
    for n, val in zip(field.dofnums, field.dofvals):
        for j in range(field.ncomp):
            v[n[j] - 1] = val[j]
    return v


# ---------------------------------------------------------------- assembly
def sparse(I, J, V, m, n):
    """SparseArrays.sparse(I, J, V, m, n) semantics; I, J 0-based int64."""
    I = np.ascontiguousarray(I, dtype=np.int64)
    J = np.ascontiguousarray(J, dtype=np.int64)
    V = np.ascontiguousarray(V, dtype=np.float64)
    k = I.shape[0]
    colptr = np.zeros(n + 1, dtype=np.int64)
    rowval = np.zeros(max(k, 1), dtype=np.int64)
    nzval = np.zeros(max(k, 1), dtype=np.float64)
    nnz = lib().oracle_sparse(ctypes.c_int64(k), _p(I, _i64), _p(J, _i64), _p(V), ctypes.c_int64(m),
                              ctypes.c_int64(n), _p(colptr, _i64), _p(rowval, _i64), _p(nzval))
    return sp.csc_matrix((nzval[:nnz].copy(), rowval[:nnz].copy(), colptr), shape=(m, n))


def local_coo(edofs_r, edofs_c, ke):
    """Triplets of LocalMatrixAssembler.init! + assemble! (column-major).

    edofs_r: (E, nr) 0-based, edofs_c: (E, nc) 0-based, ke: (E, nr*nc) column-major.
    Returns flat I, J, V in append order (element-major).
    """
    E, nr = edofs_r.shape
    nc = edofs_c.shape[1]
    I = np.repeat(edofs_r[:, None, :], nc, axis=1).reshape(E, nr * nc)  # i fastest
    J = np.repeat(edofs_c[:, :, None], nr, axis=2).reshape(E, nr * nc)
    return I.ravel(), J.ravel(), ke.reshape(E, nr * nc).ravel()


def local_coo_transpose(edofs_r, edofs_c, ke):
    """assemble!(a, transpose(lma)) of src/Assemblers.jl:109-114.

    The reference appends transpose(parent.col), transpose(parent.row) and
    transpose(parent.M), i.e. the parent's entries in row-major order with the
    row and column numbers swapped.
    """
    E, nr = edofs_r.shape
    nc = edofs_c.shape[1]
    M = ke.reshape(E, nc, nr)  # [e, j, i] = ke[i + j*nr]
    V = M.transpose(0, 2, 1)  # [e, i, j], i outer / j inner
    I = np.repeat(edofs_c[:, None, :], nr, axis=1)  # cdofs[j]
    J = np.repeat(edofs_r[:, :, None], nc, axis=2)  # rdofs[i]
    return I.ravel(), J.ravel(), V.reshape(-1)


def vec_assemble(n, edofs, fe):
    """SysvecAssembler: F[gi] += fe[i], element by element (Assemblers.jl:215-221)."""
    F = np.zeros(n)
    # np.add.at processes indices in order, so duplicates sum in element order
    np.add.at(F, edofs.ravel(), fe.ravel())
    return F


def heat_element_matrices(nn, npts, conn0, xy, kappa, Q):
    pc, w = quadrature_triangle(npts)
    N, G = bfun_tables(nn, pc)
    E = conn0.shape[0]
    conn0 = np.ascontiguousarray(conn0, dtype=np.int64)
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    kappa = np.ascontiguousarray(np.broadcast_to(np.asarray(kappa, dtype=np.float64), (E,)))
    ke = np.zeros((E, nn * nn))
    fe = np.zeros((E, nn))
    lib().oracle_heat(nn, npts, _p(N), _p(G), _p(w), ctypes.c_int64(E), _p(conn0, _i64), _p(xy),
                      _p(kappa), ctypes.c_double(Q), _p(ke), _p(fe))
    return ke, fe


def assemble_heat(nn, npts, conn0, xy, edofs0, ndofs, kappa, Q):
    """assembleKF of test/test_heat.jl:35-71: returns (K csc, F)."""
    ke, fe = heat_element_matrices(nn, npts, conn0, xy, kappa, Q)
    I, J, V = local_coo(edofs0, edofs0, ke)
    K = sparse(I, J, V, ndofs, ndofs)
    F = vec_assemble(ndofs, edofs0, fe)
    return K, F


def elasticity_element_matrices(npts, conn0, xy, D, bforce=None):
    nn = conn0.shape[1]
    pc, w = quadrature_triangle(npts)
    N, G = bfun_tables(nn, pc)
    E = conn0.shape[0]
    nd = 2 * nn
    conn0 = np.ascontiguousarray(conn0, dtype=np.int64)
    D = np.ascontiguousarray(D, dtype=np.float64)
    ke = np.zeros((E, nd * nd))
    fe = np.zeros((E, nd))
    bf = None if bforce is None else np.ascontiguousarray(bforce, dtype=np.float64)
    lib().oracle_elasticity(nn, npts, _p(N), _p(G), _p(w), ctypes.c_int64(E), _p(conn0, _i64),
                            _p(np.ascontiguousarray(xy, dtype=np.float64)), _p(D),
                            _p(bf) if bf is not None else None, _p(ke), _p(fe))
    return ke, fe


def stokes_veclap_element_matrices(npts, uconn0, xy, mu):
    pc, w = quadrature_triangle(npts)
    Nu, Gu = bfun_tables(6, pc)
    Np, _ = bfun_tables(3, pc)
    E = uconn0.shape[0]
    kuu = np.zeros((E, 144))
    kup = np.zeros((E, 36))
    lib().oracle_stokes_veclap(npts, _p(Nu), _p(Gu), _p(Np), _p(w), ctypes.c_int64(E),
                               _p(np.ascontiguousarray(uconn0, dtype=np.int64), _i64),
                               _p(np.ascontiguousarray(xy, dtype=np.float64)), ctypes.c_double(mu),
                               _p(kuu), _p(kup))
    return kuu, kup


def stokes_reddy_element_matrices(npts, uconn0, pconn0, uxy, pxy, mu):
    pc, w = quadrature_triangle(npts)
    Nu, Gu = bfun_tables(6, pc)
    Np, Gp = bfun_tables(3, pc)
    E = uconn0.shape[0]
    out = [np.zeros((E, 36)) for _ in range(3)] + [np.zeros((E, 18)) for _ in range(2)]
    lib().oracle_stokes_reddy(npts, _p(Gu), _p(Gp), _p(Np), _p(w), ctypes.c_int64(E),
                              _p(np.ascontiguousarray(uconn0, dtype=np.int64), _i64),
                              _p(np.ascontiguousarray(pconn0, dtype=np.int64), _i64),
                              _p(np.ascontiguousarray(uxy, dtype=np.float64)),
                              _p(np.ascontiguousarray(pxy, dtype=np.float64)), ctypes.c_double(mu),
                              *[_p(o) for o in out])
    return out


# ---------------------------------------------------------------- solve
def solve_lifted(K, F, T, nu):
    """solve! of test/test_heat.jl:73-76 with SuperLU in place of SuiteSparse."""
    T = np.array(T, dtype=np.float64)
    KT = K @ T
    A = K[:nu, :nu].tocsc()
    T[:nu] = spla.spsolve(A, F[:nu] - KT[:nu])
    return T


def pcg(A, b, rtol=1e-10, maxit=100000, x0=None, threads=0):
    """FP64 Jacobi-PCG (C).  A: scipy sparse (symmetric), b: rhs."""
    A = sp.csr_matrix(A)
    n = A.shape[0]
    rp = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(A.indices, dtype=np.int64)
    v = np.ascontiguousarray(A.data, dtype=np.float64)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    rr = ctypes.c_double(0)
    if threads:
        lib().oracle_set_threads(threads)
    it = lib().oracle_pcg(ctypes.c_int64(n), _p(rp, _i64), _p(ci, _i64), _p(v), _p(b), _p(x),
                          ctypes.c_double(rtol), ctypes.c_int(maxit), ctypes.byref(rr))
    return x, it, rr.value


# ---------------------------------------------------------------- errors
def l2_error_scalar(conn0, xy, nn, vals_by_node, exact, npts=3):
    """evaluate_pressure_error of test/test_stokes.jl:438-462 for an nn-node field."""
    pc, w = quadrature_triangle(npts)
    N, G = bfun_tables(nn, pc)
    X = xy[conn0]  # E x nn x 2
    E2 = 0.0
    for q in range(len(w)):
        J = np.einsum("ena,nb->eab", X, G[q])
        det = J[:, 0, 0] * J[:, 1, 1] - J[:, 1, 0] * J[:, 0, 1]
        loc = np.einsum("ena,n->ea", X, N[q])
        ua = vals_by_node[conn0] @ N[q]
        E2 += np.sum(det * w[q] * (ua - exact(loc[:, 0], loc[:, 1])) ** 2)
    return float(np.sqrt(E2))


def l2_error_vector(conn0, xy, nn, ux_by_node, uy_by_node, exx, exy, npts=3):
    """evaluate_velocity_error of test/test_stokes.jl:464-496 / 716-746."""
    pc, w = quadrature_triangle(npts)
    N, G = bfun_tables(nn, pc)
    X = xy[conn0]
    E2 = 0.0
    for q in range(len(w)):
        J = np.einsum("ena,nb->eab", X, G[q])
        det = J[:, 0, 0] * J[:, 1, 1] - J[:, 1, 0] * J[:, 0, 1]
        loc = np.einsum("ena,n->ea", X, N[q])
        ua = ux_by_node[conn0] @ N[q]
        va = uy_by_node[conn0] @ N[q]
        E2 += np.sum(det * w[q] * ((ua - exx(loc[:, 0], loc[:, 1])) ** 2 + (va - exy(loc[:, 0], loc[:, 1])) ** 2))
    return float(np.sqrt(E2))


def set_threads(n):
    lib().oracle_set_threads(int(n))


def num_threads():
    return int(lib().oracle_num_threads())
