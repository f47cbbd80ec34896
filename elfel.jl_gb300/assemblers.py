"""System matrix / vector assemblers backed by the GB300 library.

``SysmatAssemblerSparse`` and ``SysvecAssembler`` keep the reference's API
(Elfel.jl src/Assemblers.jl): ``start``/``assemble``/``finish``, with
``finish`` returning a CSC matrix (scipy.sparse.csc_matrix, Int64 indices) /
a dense vector.  Triplets are appended on the host as the reference does;
``finish`` moves them to the device, where the CSC is built and duplicates
are summed in append order (SparseArrays.sparse semantics).

``SysmatAssemblerGPU`` is the fused form: the element loop of the user's
``integrate!`` for heat, elasticity or Stokes runs on the device, the pattern
is built once and kept, and K and F stay resident for ``solve``.
"""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _native as N
from .feiterators import FEIterator, QPIterator
from .local_assemblers import LocalMatrixAssembler, LocalVectorAssembler, Transpose


class _Handle:
    def __init__(self, ctx):
        self.ctx = ctx or N.default_context()
        self.lib = self.ctx.lib
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.elfel_sysmat_create(self.ctx.h, ctypes.byref(h)))
        self.h = h
        self.ctx.adopt(self)

    def close(self):
        # a system never outlives its context: Context.close() closes it first
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.lib.elfel_sysmat_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        self.ctx.check(rc)

    def csc(self):
        nr, nc, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self.check(self.lib.elfel_sysmat_dims(self.h, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(nnz)))
        colptr = np.empty(nc.value + 1, dtype=np.int64)
        rowval = np.empty(max(nnz.value, 1), dtype=np.int64)
        nzval = np.empty(max(nnz.value, 1), dtype=np.float64)
        self.check(self.lib.elfel_sysmat_csc(self.h, N.ptr(colptr, N._i64p), N.ptr(rowval, N._i64p), N.ptr(nzval)))
        k = nnz.value
        # 1-based SparseMatrixCSC arrays -> 0-based scipy CSC (indices kept Int64)
        return sp.csc_matrix((nzval[:k], rowval[:k] - 1, colptr - 1), shape=(nr.value, nc.value))


class SysmatAssemblerSparse:
    """Sparse system matrix assembler (src/Assemblers.jl:19-123), device CSC build."""

    def __init__(self, zero=0.0, ctx=None):
        self._ctx = ctx
        self._hd = None
        self.nrow = self.ncol = 0
        self._chunks = []
        self._scalar = ([], [], [])

    def _flush_scalars(self):
        r, c, v = self._scalar
        if r:
            self._chunks.append((np.array(r, dtype=np.int64), np.array(c, dtype=np.int64),
                                 np.array(v, dtype=np.float64)))
            self._scalar = ([], [], [])

    def triplets(self):
        """The appended (row, col, val) triplets, 1-based, in append order."""
        self._flush_scalars()
        if not self._chunks:
            return (np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0))
        return tuple(np.concatenate([ch[k] for ch in self._chunks]) for k in range(3))


def start(a, nrow, ncol=None):
    """start!(assembler, nrow, ncol) / start!(vector assembler, nrow)."""
    if isinstance(a, SysmatAssemblerSparse):
        a.nrow, a.ncol = int(nrow), int(ncol)
        a._chunks = []
        a._scalar = ([], [], [])
        return a
    if isinstance(a, SysvecAssembler):
        a.ndofs = int(nrow)
        a._rows, a._vals = [], []
        return a
    if isinstance(a, SysmatAssemblerGPU):
        a.nrow, a.ncol = int(nrow), int(ncol)
        return a
    raise TypeError(type(a))


def assemble(a, *args):
    """assemble!(a, r, c, v) | assemble!(a, lma) | assemble!(a, transpose(lma)) |
    assemble!(av, i, v) | assemble!(av, lva)   (src/Assemblers.jl:85-114, 205-221)."""
    if isinstance(a, SysmatAssemblerSparse):
        if len(args) == 3:
            a._scalar[0].append(int(args[0]))
            a._scalar[1].append(int(args[1]))
            a._scalar[2].append(float(args[2]))
            return a
        lma = args[0]
        a._flush_scalars()
        if isinstance(lma, Transpose):
            p = lma.parent  # parent entries row-major, row/col swapped (Assemblers.jl:109-114)
            a._chunks.append((p.col.ravel(order="C").copy(), p.row.ravel(order="C").copy(),
                              p.M.ravel(order="C").copy()))
        elif isinstance(lma, LocalMatrixAssembler):
            a._chunks.append((lma.row.ravel(order="F").copy(), lma.col.ravel(order="F").copy(),
                              lma.M.ravel(order="F").copy()))
        else:
            raise TypeError(type(lma))
        return a
    if isinstance(a, SysvecAssembler):
        if len(args) == 2:
            a._rows.append(np.array([int(args[0])], dtype=np.int64))
            a._vals.append(np.array([float(args[1])]))
        else:
            lva = args[0]
            if not isinstance(lva, LocalVectorAssembler):
                raise TypeError(type(lva))
            a._rows.append(lva.row.copy())
            a._vals.append(lva.V.copy())
        return a
    raise TypeError(type(a))


def finish(a):
    """finish!(a): CSC matrix (SysmatAssemblerSparse) or dense vector (SysvecAssembler)."""
    if isinstance(a, SysmatAssemblerSparse):
        I, J, V = a.triplets()
        if a._hd is None:
            a._hd = _Handle(a._ctx)
        h = a._hd
        h.check(h.lib.elfel_sysmat_start(h.h, a.nrow, a.ncol))
        n = I.shape[0]
        h.check(h.lib.elfel_sysmat_assemble_coo(h.h, N.ptr(I, N._i64p), N.ptr(J, N._i64p), N.ptr(V), n))
        nnz = ctypes.c_int64()
        h.check(h.lib.elfel_sysmat_finish(h.h, ctypes.byref(nnz)))
        return h.csc()
    if isinstance(a, SysvecAssembler):
        ctx = a._ctx or N.default_context()
        rows = np.concatenate(a._rows) if a._rows else np.zeros(0, np.int64)
        vals = np.concatenate(a._vals) if a._vals else np.zeros(0)
        out = np.zeros(a.ndofs)
        ctx.check(ctx.lib.elfel_sysvec_assemble(ctx.h, a.ndofs, N.ptr(rows, N._i64p), N.ptr(vals), rows.shape[0],
                                                N.ptr(out)))
        return out
    if isinstance(a, SysmatAssemblerGPU):
        return a.csc()
    raise TypeError(type(a))


class SysvecAssembler:
    """Dense system vector assembler (src/Assemblers.jl:170-230), device summation."""

    def __init__(self, zero=0.0, ctx=None):
        self._ctx = ctx
        self.ndofs = 0
        self._rows, self._vals = [], []


# ---------------------------------------------------------------- fused form
_SOLVERS = {"pcg64": N.ELFEL_PCG64, "pcg32_ir": N.ELFEL_PCG32_IR, "minres64": N.ELFEL_MINRES64,
            "minres32_ir": N.ELFEL_MINRES32_IR}


def _shape_of(fesp):
    """(enum elfel_shape, coordinates per node) of a space the fused kernels take."""
    from . import felements as fel

    fe = fesp.fe
    if type(fe) in (fel.FEH1_T3, fel.FEH1_T6):
        return N.ELFEL_SHAPE_TRIANGLE, 2
    if type(fe) is fel.FEH1_Q4:
        return N.ELFEL_SHAPE_Q4, 2
    if type(fe) is fel.FEH1_T4:
        return N.ELFEL_SHAPE_T4, 3
    raise N.ElfelError(N.ELFEL_ERR_UNSUPPORTED, f"fused device assembly takes FEH1_T3, FEH1_T6, FEH1_Q4 and FEH1_T4 "
                                                f"spaces, not {fe}: assemble it with SysmatAssemblerSparse")


def _space_struct(elit: FEIterator, keep):
    fesp = elit.fesp
    mesh = fesp.mesh
    conn = N.i64(mesh.conn)
    xy = N.f64(mesh.xy)
    dofs = N.i64(elit.eldofs_table())
    keep.extend([conn, xy, dofs])
    return N.Space(mesh.nodes_per_elem, fesp.nfecopies, mesh.nel, mesh.nnodes, N.ptr(conn, N._i64p), N.ptr(xy),
                   N.ptr(dofs, N._i64p))


class SysmatAssemblerGPU:
    """Fused device assembler: the element loop runs on the GPU.

    Usage mirrors the reference scripts::

        am = start(SysmatAssemblerGPU(), ndofs(fesp), ndofs(fesp))
        assemble_heat(am, FEIterator(fesp), QPIterator(fesp, {"npts": 3}), kappa, Q)
        K = finish(am); F = am.rhs()
        solve(T, am, None, nunknowns(fesp), method="pcg32_ir")
    """

    def __init__(self, ctx=None):
        self._hd = _Handle(ctx)
        self.nrow = self.ncol = 0
        self._setup_key = None
        self._keep = []
        self.physics = None

    @property
    def ctx(self):
        return self._hd.ctx

    def setup(self, physics, elit, qpit, pelit=None, ndofs=None):
        """Upload the mesh and DOF tables and build the pattern once."""
        keep = []
        u = _space_struct(elit, keep)
        p = _space_struct(pelit, keep) if pelit is not None else N.Space()
        qr = qpit.quadr
        pc = N.f64(qr.param_coords)
        w = N.f64(qr.weights)
        keep.extend([pc, w])
        n = int(ndofs if ndofs is not None else self.nrow)
        shape, sdim = _shape_of(elit.fesp)
        d = N.FusedDesc(physics, qr.npts, N.ptr(pc), N.ptr(w), n, u, p, shape, sdim)
        self._hd.check(self._hd.lib.elfel_fused_setup(self._hd.h, ctypes.byref(d)))
        self._keep = keep
        self.physics = physics
        self.nrow = self.ncol = n
        self.nel = elit.fesp.mesh.nel
        self._nn = elit.fesp.mesh.nodes_per_elem
        self._nedof = self._nn * elit.fesp.nfecopies
        self._sdim = sdim
        self._setup_key = (id(elit.fesp), id(pelit.fesp) if pelit is not None else None, qr.npts, physics, n)
        return self

    def setup_numbered(self, physics, fesp, qpit, pfesp=None):
        """Set-up with numberdofs! on the device (elfel_fused_setup_numbered):
        only the connectivity, the coordinates and the essential-BC masks
        (one byte per DOF) are uploaded; the DOF numbers come back into the
        spaces' FEFields (as numberdofs!(fesp) or numberdofs!([fesp, pfesp])
        would set them) and the element DOF tables are built on the device.
        Returns the number of unknowns."""
        spaces = [fesp] + ([pfesp] if pfesp is not None else [])
        keep, structs, masks, nums = [], [], [], []
        for sp in spaces:
            if list(sp._fields) != [0]:
                raise N.ElfelError(N.ELFEL_ERR_UNSUPPORTED, "device numbering takes spaces with nodal DOFs only")
            mesh = sp.mesh
            conn, xy = N.i64(mesh.conn), N.f64(mesh.xy)
            mask = np.ascontiguousarray(sp.field.isdatum, dtype=np.uint8)
            keep.extend([conn, xy, mask])
            structs.append(N.Space(mesh.nodes_per_elem, sp.nfecopies, mesh.nel, mesh.nnodes, N.ptr(conn, N._i64p),
                                   N.ptr(xy), None))
            masks.append(mask)
            nums.append(np.zeros(sp.field.dofnums.shape, dtype=np.int64))
        qr = qpit.quadr
        pc, w = N.f64(qr.param_coords), N.f64(qr.weights)
        keep.extend([pc, w])
        n = sum(sp.field.dofnums.size for sp in spaces)
        shape, sdim = _shape_of(fesp)
        d = N.FusedDesc(physics, qr.npts, N.ptr(pc), N.ptr(w), n, structs[0],
                        structs[1] if len(structs) > 1 else N.Space(), shape, sdim)
        nfree = ctypes.c_int64()
        self._hd.check(self._hd.lib.elfel_fused_setup_numbered(
            self._hd.h, ctypes.byref(d), masks[0].ctypes.data_as(ctypes.c_void_p),
            masks[1].ctypes.data_as(ctypes.c_void_p) if len(masks) > 1 else None, N.ptr(nums[0], N._i64p),
            N.ptr(nums[1], N._i64p) if len(nums) > 1 else None, ctypes.byref(nfree)))
        for sp, nm in zip(spaces, nums):
            sp.field.dofnums = nm
        self._keep = keep
        self.physics = physics
        self.nrow = self.ncol = n
        self.nel = fesp.mesh.nel
        self._nn = fesp.mesh.nodes_per_elem
        self._nedof = self._nn * fesp.nfecopies
        self._sdim = sdim
        self._setup_key = (id(fesp), id(pfesp) if pfesp is not None else None, qr.npts, physics, n)
        return nfree.value

    def setup_block(self, etype, nx, ny, lx=1.0, ly=1.0, orientation="a", npts=3):
        """Heat set-up from a block mesh generated on the device (T3block /
        T6block of [0,lx] x [0,ly], boundary fixed, numberdofs! order).
        Returns (ndofs, nunknowns)."""
        from .refshapes import quadrature

        qr = quadrature(quadraturesettings={"npts": npts})
        pc, w = N.f64(qr.param_coords), N.f64(qr.weights)
        d = N.BlockDesc(3 if etype == "T3" else 6, {"a": 0, "alternate": 1}[orientation], int(nx), int(ny),
                        float(lx), float(ly), int(npts), 0, N.ptr(pc), N.ptr(w))
        n, nu = ctypes.c_int64(), ctypes.c_int64()
        self._hd.check(self._hd.lib.elfel_fused_setup_block(self._hd.h, ctypes.byref(d), ctypes.byref(n),
                                                            ctypes.byref(nu)))
        self.physics = N.ELFEL_HEAT
        self.nrow = self.ncol = n.value
        self.nel = 2 * int(nx) * int(ny)
        self._nn = self._nedof = 3 if etype == "T3" else 6
        self._sdim = 2
        self._setup_key = ("block", etype, nx, ny, lx, ly, orientation, npts)
        return n.value, nu.value

    def block_dirichlet(self, coef):
        """T (ndofs): 0 at free DOFs, c0 + c1 x + c2 y + c3 x^2 + c4 x y + c5 y^2 at data DOFs."""
        c = N.f64(np.asarray(coef, dtype=np.float64).reshape(6))
        T = np.empty(self.nrow)
        self._hd.check(self._hd.lib.elfel_block_dirichlet(self._hd.h, N.ptr(c), N.ptr(T)))
        return T

    def tables(self):
        """(conn, xy, eldofs) of the fused system, 1-based as the set-up takes them."""
        nel, nnodes, nd = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._hd.check(self._hd.lib.elfel_fused_dims(self._hd.h, ctypes.byref(nel), ctypes.byref(nnodes),
                                                     ctypes.byref(nd)))
        conn = np.empty((nel.value, self._nn), dtype=np.int64)
        dofs = np.empty((nel.value, self._nedof), dtype=np.int64)
        xy = np.empty((nnodes.value, self._sdim))
        self._hd.check(self._hd.lib.elfel_fused_tables(self._hd.h, N.ptr(conn, N._i64p), N.ptr(xy),
                                                       N.ptr(dofs, N._i64p)))
        return conn, xy, dofs

    def error_l2(self, U, exact, space=0, npts=3):
        """evaluate_pressure_error / evaluate_velocity_error of test/test_stokes.jl:438-496
        on the device: the L2 norm of u_h - u_exact over space 0 (primary) or 1
        (Taylor-Hood pressure).  exact: one dict {(a, b): c} per component, the
        polynomial sum c x^a y^b of degree <= 4."""
        from .refshapes import quadrature

        if isinstance(exact, dict):
            exact = [exact]
        poly = np.zeros((len(exact), 15))
        order = [(a, d - a) for d in range(5) for a in range(d, -1, -1)]
        for k, terms in enumerate(exact):
            for (a, b), v in terms.items():
                poly[k, order.index((a, b))] = v
        qr = quadrature(quadraturesettings={"npts": npts})
        pc, w = N.f64(qr.param_coords), N.f64(qr.weights)
        U = N.f64(U)
        poly = N.f64(poly)
        e = ctypes.c_double()
        self._hd.check(self._hd.lib.elfel_error_l2(self._hd.h, N.ptr(U), int(space), N.ptr(poly), int(npts),
                                                   N.ptr(pc), N.ptr(w), ctypes.byref(e)))
        return e.value

    def _ensure(self, physics, elit, qpit, pelit=None):
        key = (id(elit.fesp), id(pelit.fesp) if pelit is not None else None, qpit.quadr.npts, physics, self.nrow)
        if key != self._setup_key:
            self.setup(physics, elit, qpit, pelit)

    def heat(self, kappa, Q):
        """K and F of the heat weak form; kappa: scalar, per-element array, or None (resident)."""
        if kappa is not None:
            kappa = np.ascontiguousarray(np.broadcast_to(np.asarray(kappa, dtype=np.float64), (self.nel,)))
        self._hd.check(self._hd.lib.elfel_fused_heat(self._hd.h, N.ptr(kappa), float(Q)))
        return self

    def elasticity(self, E, nu, plane_strain=True, bforce=None, trac_edges=None, traction=(0.0, 0.0)):
        bf = N.f64(bforce) if bforce is not None else None
        te = N.i64(trac_edges) if trac_edges is not None else None
        tr = N.f64(traction)
        nt = 0 if te is None else te.shape[0]
        self._hd.check(self._hd.lib.elfel_fused_elasticity(self._hd.h, float(E), float(nu), int(bool(plane_strain)),
                                                           N.ptr(bf), N.ptr(te, N._i64p), nt, N.ptr(tr)))
        return self

    def stokes(self, mu):
        self._hd.check(self._hd.lib.elfel_fused_stokes(self._hd.h, float(mu)))
        return self

    def tile_stats(self):
        """(tiles, distinct tile programs, tiles on the contributor-list path, runs of tiles of one
        program) of the K pattern's tile reduction plan; zeros before the plan is built."""
        a, b, c, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._hd.check(self._hd.lib.elfel_sysmat_tile_stats(self._hd.h, ctypes.byref(a), ctypes.byref(b),
                                                            ctypes.byref(c), ctypes.byref(d)))
        return a.value, b.value, c.value, d.value

    def set_geometry(self, xy):
        xy = N.f64(xy)
        self._hd.check(self._hd.lib.elfel_fused_set_geometry(self._hd.h, N.ptr(xy)))

    def csc(self):
        return self._hd.csc()

    def rhs(self):
        F = np.zeros(self.nrow)
        self._hd.check(self._hd.lib.elfel_sysmat_rhs(self._hd.h, N.ptr(F)))
        return F

    def solve(self, T, nu, F=None, method="pcg32_ir", rtol=1e-10, maxit=200000):
        """solve!(T, K, F, nu) of test/test_heat.jl:73-76, on the device.  T is updated in place."""
        return _solve_handle(self._hd, T, nu, F, method, rtol, maxit)


def numberdofs_device(fesp, ctx=None):
    """numberdofs!(fesp) / numberdofs!([fesp1, fesp2, ...]) (src/FESpaces.jl:250-259)
    computed on the device (elfel_number_dofs) from the spaces' essential-BC
    masks; the numbers are written into the spaces' fields.  Returns the
    number of unknowns.  Spaces with nodal DOFs only."""
    spaces = list(fesp) if isinstance(fesp, (list, tuple)) else [fesp]
    ctx = ctx or N.default_context()
    for sp in spaces:
        if list(sp._fields) != [0]:
            raise N.ElfelError(N.ELFEL_ERR_UNSUPPORTED, "device numbering takes spaces with nodal DOFs only")
    ns = len(spaces)
    masks = [np.ascontiguousarray(sp.field.isdatum, dtype=np.uint8) for sp in spaces]
    nums = [np.zeros(sp.field.dofnums.shape, dtype=np.int64) for sp in spaces]
    nterms = (ctypes.c_int64 * ns)(*[sp.field.dofnums.shape[0] for sp in spaces])
    ncomp = (ctypes.c_int32 * ns)(*[sp.field.dofnums.shape[1] for sp in spaces])
    mp = (ctypes.c_void_p * ns)(*[m.ctypes.data_as(ctypes.c_void_p).value for m in masks])
    np_ = (N._i64p * ns)(*[N.ptr(x, N._i64p) for x in nums])
    nfree = ctypes.c_int64()
    ctx.check(ctx.lib.elfel_number_dofs(ctx.h, ns, nterms, ncomp, mp, np_, ctypes.byref(nfree)))
    for sp, nm in zip(spaces, nums):
        sp.field.dofnums = nm
    return nfree.value


def assemble_heat(am, elit, qpit, kappa, Q):
    """Fused integrate! of test/test_heat.jl:36-60: K and F on the device."""
    am._ensure(N.ELFEL_HEAT, elit, qpit)
    return am.heat(kappa, Q)


def assemble_elasticity(am, elit, qpit, E, nu, plane_strain=True, bforce=None, trac_edges=None,
                        traction=(0.0, 0.0)):
    """Fused integrateK! of test/test_elasticity.jl:150-171 plus loads."""
    am._ensure(N.ELFEL_ELASTICITY, elit, qpit)
    return am.elasticity(E, nu, plane_strain, bforce, trac_edges, traction)


def assemble_stokes(am, uelit, pelit, qpit, mu):
    """Fused integrate! of test/test_stokes.jl:629-657 (vector Laplacian Taylor-Hood)."""
    am._ensure(N.ELFEL_STOKES, uelit, qpit, pelit)
    return am.stokes(mu)


def _solve_handle(hd, T, nu, F, method, rtol, maxit):
    st = N.SolveStats()
    Fa = N.f64(F) if F is not None else None
    if T.dtype != np.float64 or not T.flags.c_contiguous:
        raise TypeError("T must be a contiguous float64 array")
    rc = hd.lib.elfel_solve(hd.h, N.ptr(Fa), N.ptr(T), int(nu), _SOLVERS[method], float(rtol), int(maxit),
                            ctypes.byref(st))
    stats = st.as_dict()
    hd.check(rc)
    return stats


def solve(T, K, F, nu, method="pcg32_ir", rtol=1e-10, maxit=200000, ctx=None):
    """solve!(T, K, F, nu): T[1:nu] = K[1:nu,1:nu] \\ (F - K*T)[1:nu] on the device.

    K is the device-resident fused system (SysmatAssemblerGPU; F may be None),
    a finished SysmatAssemblerSparse, or any host sparse matrix (uploaded).
    T is updated in place; returns the solver statistics.
    """
    if isinstance(K, SysmatAssemblerGPU):
        return K.solve(T, nu, F, method, rtol, maxit)
    if F is None:
        raise ValueError("F is required unless K is a fused device system")
    if isinstance(K, SysmatAssemblerSparse):
        if K._hd is None:
            raise ValueError("finish the assembler before solving")
        return _solve_handle(K._hd, T, nu, F, method, rtol, maxit)
    A = sp.coo_matrix(K)
    a = start(SysmatAssemblerSparse(0.0, ctx=ctx), A.shape[0], A.shape[1])
    a._chunks.append((A.row.astype(np.int64) + 1, A.col.astype(np.int64) + 1, A.data.astype(np.float64)))
    finish(a)
    return _solve_handle(a._hd, T, nu, F, method, rtol, maxit)
