"""Device assembly against the oracle (GPU).

Pattern (colptr/rowval) and DOF numbering: bit-exact.  Values: FP64, within
1e-12 of the largest entry (the device reorganises the quadrature sums of
straight-sided elements, so the last bits differ).  COO mode sums in the same
order as the oracle and is checked bit for bit.
"""
import numpy as np
import pytest

from problems import (elasticity_D, elasticity_setup, heat_oracle, heat_space, stokes_oracle_K, stokes_setup,
                      traction_oracle)

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # FP64 parity tolerance, relative to max |entry|


def same_pattern(K, K0):
    K.sort_indices()
    return (K.indptr == K0.indptr).all() and (K.indices == K0.indices).all() and K.shape == K0.shape


def close(a, b, rtol=RTOL):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= rtol * scale


def test_coo_7x7_golden(E, O, gpu, golden):
    """test/test_assemblers.jl:6-34 through SysmatAssemblerSparse on the device."""
    g = golden("assemblers.json")
    a = E.start(E.SysmatAssemblerSparse(0.0), 7, 7)
    for blk in g["blocks"]:
        m = np.array(blk["m"])
        for j in range(m.shape[1]):
            for i in range(m.shape[0]):
                E.assemble(a, blk["gi"][i], blk["gj"][j], m[i, j])
    A = E.finish(a)
    B = np.array(g["B"])
    assert np.linalg.norm(A.toarray() - B) / np.linalg.norm(B) < g["rtol"]
    I, J, V = a.triplets()
    A0 = O.sparse(I - 1, J - 1, V, 7, 7)
    assert same_pattern(A, A0) and (A.data == A0.data).all()


def test_coo_local_and_transpose(E, O, gpu, golden):
    """test/test_assemblers.jl:47-129: local assemblers, plain and transposed."""
    g = golden("assemblers.json")
    B = np.array(g["B"])
    for transposed in (False, True):
        a = E.start(E.SysmatAssemblerSparse(0.0), 7, 7)
        for blk in g["blocks"]:
            m = np.array(blk["m"])
            gi, gj = blk["gi"], blk["gj"]
            if transposed:
                la = E.LocalMatrixAssembler(len(gj), len(gi), 0.0)
                E.init(la, gj, gi)
                la.M[:, :] = m.T
                E.assemble(a, E.transpose(la))
            else:
                la = E.LocalMatrixAssembler(len(gi), len(gj), 0.0)
                E.init(la, gi, gj)
                la.M[:, :] = m
                E.assemble(a, la)
        A = E.finish(a).toarray()
        assert np.linalg.norm(A - B) / np.linalg.norm(B) < g["rtol"]


@pytest.mark.parametrize("seed,n,m,k", [(0, 50, 40, 3000), (1, 1, 1, 10), (2, 300, 7, 20000), (3, 5, 2000, 4000)])
def test_coo_random_bitexact(E, O, gpu, seed, n, m, k):
    """Random triplets with many duplicates, zeros, a long column: bit-exact vs the oracle."""
    rng = np.random.default_rng(seed)
    I = rng.integers(1, n + 1, k)
    J = rng.integers(1, m + 1, k)
    if m > 3:
        J[: k // 3] = 2  # one long column (> one warp's shared-memory tile)
    V = rng.standard_normal(k)
    V[::5] = 0.0
    a = E.start(E.SysmatAssemblerSparse(0.0), n, m)
    a._chunks.append((I, J, V))
    A = E.finish(a)
    A0 = O.sparse(I - 1, J - 1, V, n, m)
    assert same_pattern(A, A0)
    assert (A.data == A0.data).all()


def test_coo_empty_and_errors(E, gpu):
    a = E.start(E.SysmatAssemblerSparse(0.0), 4, 3)
    A = E.finish(a)
    assert A.shape == (4, 3) and A.nnz == 0
    a = E.start(E.SysmatAssemblerSparse(0.0), 4, 3)
    E.assemble(a, 5, 1, 1.0)  # row outside 1..4
    with pytest.raises(E.ElfelError):
        E.finish(a)


def test_sysvec(E, gpu):
    """test/test_assemblers.jl:142-163 (SysvecAssembler)."""
    rng = np.random.default_rng(5)
    N = 30
    v = np.zeros(N)
    a = E.start(E.SysvecAssembler(), N)
    for rows in ([1, 7, 2], [29, 15, 1, 7, 3, 6, 2]):
        vals = rng.random(len(rows))
        for i, p in zip(rows, vals):
            E.assemble(a, i, p)
            v[i - 1] += p
    w = E.finish(a)
    assert np.linalg.norm(v - w) / np.linalg.norm(w) <= 1e-9
    lva = E.LocalVectorAssembler(3, 0.0)
    E.init(lva, [3, 3, 1])
    lva.V[:] = [1.0, 2.0, 4.0]
    a = E.start(E.SysvecAssembler(), 4)
    E.assemble(a, lva)
    assert E.finish(a).tolist() == [4.0, 0.0, 3.0, 0.0]


HEAT_CASES = [
    # etype, nx, ny, orientation, jitter, curved, npts
    ("T3", 4, 4, "a", 0.0, False, 1),
    ("T3", 17, 9, "alternate", 0.02, False, 3),
    ("T6", 6, 5, "a", 0.0, False, 3),
    ("T6", 13, 11, "alternate", 0.02, False, 3),
    ("T6", 9, 7, "a", 0.01, True, 3),
    ("T6", 8, 8, "a", 0.01, True, 6),
    ("T3", 100, 100, "alternate", 0.0, False, 3),
    ("T6", 7, 6, "a", 0.01, False, 1),  # inexact rule: the general tensor form
    ("T6", 10, 9, "alternate", 0.02, False, 7),
]


@pytest.mark.parametrize("case", HEAT_CASES)
def test_fused_heat_parity(E, O, gpu, case):
    etype, nx, ny, orient, jit, curved, npts = case
    blk = E.T3block if etype == "T3" else E.T6block
    mesh = blk(1.0, 1.0, nx, ny, orientation=orient)
    if jit:
        mesh = E.jitter(mesh, jit / max(nx, ny), seed=11, curved=curved)
    fe = E.FEH1_T3() if etype == "T3" else E.FEH1_T6()
    fesp = heat_space(E, mesh, fe)
    rng = np.random.default_rng(4)
    kappa = np.exp(rng.uniform(np.log(0.5), np.log(2.0), mesh.nel))
    n = E.ndofs(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"kind": "default", "npts": npts}), kappa, -6.0)
    K, F = E.finish(am), am.rhs()
    K0, F0 = heat_oracle(E, O, mesh, fesp, npts, kappa, -6.0)
    assert same_pattern(K, K0)
    assert close(K.data, K0.data) and close(F, F0)
    # re-assembly with new coefficients reuses the pattern
    am.heat(kappa * 2.0, -3.0)
    K2 = E.finish(am)
    assert same_pattern(K2, K0) and close(K2.data, 2.0 * K0.data)


def test_fused_heat_nnz_formula(E, gpu):
    """Pattern size of the uniform T6 block: 46 N^2 + 16 N + 1 nonzeros."""
    for N in (3, 10, 31):
        mesh = E.T6block(1.0, 1.0, N, N)
        fesp = heat_space(E, mesh, E.FEH1_T6())
        n = E.ndofs(fesp)
        am = E.start(E.SysmatAssemblerGPU(), n, n)
        E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.0, -6.0)
        assert E.finish(am).nnz == 46 * N * N + 16 * N + 1


@pytest.mark.parametrize("etype,curved", [("T3", False), ("T6", False), ("T6", True)])
def test_fused_elasticity_parity(E, O, gpu, etype, curved):
    mesh, fesp, bforce, right = elasticity_setup(E, 10, 6, etype=etype)
    if curved:
        mesh = E.jitter(mesh, 0.01, seed=2, curved=True)
        fesp = E.FESpace(float, mesh, fesp.fe, 2)
        left = E.vselect(mesh.xy, [0.0, 0.0, 0.0, 1.0], inflate=1e-4)
        E.setebc(fesp, 0, left, 1, 0.0)
        E.setebc(fesp, 0, left, 2, 0.0)
        E.numberdofs(fesp)
    n = E.ndofs(fesp)
    elit = E.FEIterator(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_elasticity(am, elit, E.QPIterator(fesp, {"npts": 3}), 1.0, 0.3, True, bforce, right, (1.0, 0.0))
    K, F = E.finish(am), am.rhs()
    D = elasticity_D(1.0, 0.3, True)
    ke, fe = O.elasticity_element_matrices(3, mesh.conn - 1, mesh.xy, D, bforce)
    ed = elit.eldofs_table() - 1
    K0 = O.sparse(*O.local_coo(ed, ed, ke), n, n)
    F0 = O.vec_assemble(n, ed, fe)
    if not curved:
        F0 = F0 + traction_oracle(mesh, ed, right, (1.0, 0.0), n)
    assert same_pattern(K, K0)
    assert close(K.data, K0.data)
    if not curved:
        assert close(F, F0)


def test_fused_stokes_parity(E, O, gpu):
    vmesh, pmesh, ufesp, pfesp = stokes_setup(E, 6)
    K0, n = stokes_oracle_K(E, O, vmesh, ufesp, pfesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_stokes(am, E.FEIterator(ufesp), E.FEIterator(pfesp), E.QPIterator(ufesp, {"npts": 3}), 1.0)
    K = E.finish(am)
    assert same_pattern(K, K0)
    assert close(K.data, K0.data)
    # explicit zeros of the cross-component couplings are in the pattern
    assert (K.data == 0.0).sum() > 0 and (K0.data == 0.0).sum() > 0


def test_t6_straight_kernel_matches_general(E, gpu):
    """A straight-sided T6 mesh takes the straight-only kernel; the same mesh
    with one curved element takes the general kernel.  Entries away from the
    curved element must agree bit for bit (both kernels share the
    straight-sided arithmetic)."""
    mesh = E.jitter(E.T6block(1.0, 1.0, 12, 10), 0.02, seed=5)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    n = E.ndofs(fesp)
    kappa = np.linspace(0.5, 2.0, mesh.nel)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), kappa, -6.0)
    K0, F0 = E.finish(am).tocoo(), am.rhs()
    xy = mesh.xy.copy()
    e = mesh.nel // 2
    mid = mesh.conn[e, 3] - 1  # a midside node of one interior element
    xy[mid] += [1e-3, -1e-3]
    am.set_geometry(xy)
    am.heat(None, -6.0)
    K1, F1 = E.finish(am).tocoo(), am.rhs()
    touched = np.nonzero((mesh.conn - 1 == mid).any(axis=1))[0]
    dofs = E.FEIterator(fesp).eldofs_table() - 1
    near = np.zeros(n, dtype=bool)
    near[dofs[touched].ravel()] = True
    far = ~(near[K0.row] | near[K0.col])
    assert far.sum() > 0.8 * K0.nnz
    assert (K0.row == K1.row).all() and (K0.col == K1.col).all()
    assert (K0.data[far] == K1.data[far]).all()
    assert not (K0.data[~far] == K1.data[~far]).all()
    # the load vector: added by the straight-only kernel, reduced from records
    # by the general one; the same bits (signed zeros included) away from it
    assert (F0[~near].view(np.int64) == F1[~near].view(np.int64)).all()


def _phases(am, Q):
    ctx = am._hd.ctx
    ctx.profile(True)
    am.heat(None, Q)
    ph = ctx.phases()
    ctx.profile(False)
    return ph


@pytest.mark.parametrize("case", ["conforming", "mirrored_Q0", "duplicate_element"])
def test_t6_load_vector_paths(E, O, gpu, case):
    """The straight-only exact T6 kernel adds the load vector into the global
    vector when no DOF is a midside node of more than two elements (a sum of
    at most two terms onto +0 is independent of their order); otherwise the
    records go through the in-order reduction.  Both start from +0 as the
    zeroed vector of SysvecAssembler (Assemblers.jl:194-207): Q = 0 on
    clockwise elements (element loads of -0) gives +0 everywhere."""
    mesh = E.T6block(1.0, 1.0, 9, 8)
    Q = -6.0
    if case == "mirrored_Q0":
        mesh = E.Mesh("T6", mesh.conn, mesh.xy * np.array([-1.0, 1.0]))
        Q = 0.0
    if case == "duplicate_element":
        mesh = E.Mesh("T6", np.vstack([mesh.conn, mesh.conn[mesh.nel // 2]]), mesh.xy)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    n = E.ndofs(fesp)
    kappa = np.linspace(0.5, 2.0, mesh.nel)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), kappa, Q)
    ph = _phases(am, Q)
    assert ("reduce_F" in ph) == (case == "duplicate_element")
    K, F = E.finish(am), am.rhs()
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, kappa, Q)
    assert same_pattern(K, K0) and close(K.data, K0.data)
    if Q == 0.0:
        assert (F.view(np.int64) == 0).all() and (F0.view(np.int64) == 0).all()
    else:
        assert close(F, F0)


@pytest.mark.parametrize("case", ["flat", "kappa_range"])
def test_t6_pair_and_fp64_paths(E, O, gpu, case):
    """The straight-sided T6 record is evaluated in float pairs unless an
    element is strongly distorted (det J' < 1/4 after scaling) or kappa / Q
    fall outside the pair range; those take the FP64 form.  Flat elements
    (aspect ratio 40) and coefficients over 580 decades exercise the
    fallback; every entry matches the oracle to 1e-11 of its column's largest."""
    if case == "flat":
        mesh = E.jitter(E.T6block(1.0, 0.025, 8, 8), 0.0003, seed=3)
        kappa = np.linspace(0.5, 2.0, mesh.nel)
        Q = -6.0
    else:
        mesh = E.jitter(E.T6block(1.0, 1.0, 9, 7), 0.02, seed=4)
        rng = np.random.default_rng(8)
        kappa = 10.0 ** rng.uniform(-290, 290, mesh.nel)  # beyond 2^+-900 some take the FP64 form
        Q = 1e-250
    fesp = heat_space(E, mesh, E.FEH1_T6())
    n = E.ndofs(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), kappa, Q)
    K, F = E.finish(am), am.rhs()
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, kappa, Q)
    assert same_pattern(K, K0)
    # each entry against its own size (the contributions of one entry share an element scale here)
    rowmax = np.maximum.reduceat(np.abs(K0.data), K0.indptr[:-1]) if K0.nnz else np.zeros(0)
    scale = np.repeat(rowmax, np.diff(K0.indptr))
    assert (np.abs(K.data - K0.data) <= 1e-11 * scale).all()
    assert np.abs(F - F0).max() <= 1e-11 * np.abs(F0).max()


def test_fused_setup_rejects_bad_tables(E, gpu):
    """Connectivity and element DOFs are read straight from host memory and
    checked on the device; an entry outside its range fails fused_setup with
    the table's name, and the system can be set up again afterwards."""
    import ctypes

    mesh = E.T6block(1.0, 1.0, 4, 4)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    n = E.ndofs(fesp)
    qpit = E.QPIterator(fesp, {"npts": 3})
    N_ = E._native
    pc, w = N_.f64(qpit.quadr.param_coords), N_.f64(qpit.quadr.weights)
    xy = np.ascontiguousarray(mesh.xy)
    am = E.start(E.SysmatAssemblerGPU(), n, n)

    def setup(conn, dofs):
        sp = N_.Space(6, 1, mesh.nel, mesh.nnodes, N_.ptr(conn, N_._i64p), N_.ptr(xy), N_.ptr(dofs, N_._i64p))
        d = N_.FusedDesc(N_.ELFEL_HEAT, 3, N_.ptr(pc), N_.ptr(w), n, sp, N_.Space())
        am._hd.check(am._hd.lib.elfel_fused_setup(am._hd.h, ctypes.byref(d)))

    conn = np.ascontiguousarray(mesh.conn)
    dofs = np.ascontiguousarray(E.FEIterator(fesp).eldofs_table())
    bad_conn = conn.copy()
    bad_conn[5, 2] = mesh.nnodes + 1
    with pytest.raises(E.ElfelError, match="primary connectivity"):
        setup(bad_conn, dofs)
    bad_dofs = dofs.copy()
    bad_dofs[7, 1] = 0
    with pytest.raises(E.ElfelError, match="primary eldofs"):
        setup(conn, bad_dofs)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.0, -6.0)
    K, F = E.finish(am), am.rhs()
    am2 = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am2, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.0, -6.0)
    K2, F2 = E.finish(am2), am2.rhs()
    assert same_pattern(K, K2) and (K.data == K2.data).all() and (F == F2).all()


def test_fused_edge_cases(E, O, gpu):
    """One T6 element (every midside DOF with a single contribution), and a
    mesh without elements through the C ABI (empty pattern, zero vector)."""
    import ctypes

    m2 = E.T6block(1.0, 1.0, 1, 1)
    mesh = E.Mesh("T6", m2.conn[:1], m2.xy)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    n = E.ndofs(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.5, -6.0)
    K, F = E.finish(am), am.rhs()
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, np.array([1.5]), -6.0)
    assert same_pattern(K, K0) and close(K.data, K0.data) and close(F, F0)
    assert K.nnz == 36  # one element: a dense 6 x 6 block (unused nodes have empty columns)

    N_ = E._native
    qpit = E.QPIterator(fesp, {"npts": 3})
    pc, w = N_.f64(qpit.quadr.param_coords), N_.f64(qpit.quadr.weights)
    conn = np.zeros((0, 6), dtype=np.int64)
    dofs = np.zeros((0, 6), dtype=np.int64)
    xy = np.ascontiguousarray(m2.xy)
    nn = xy.shape[0]
    sp = N_.Space(6, 1, 0, nn, N_.ptr(conn, N_._i64p), N_.ptr(xy), N_.ptr(dofs, N_._i64p))
    d = N_.FusedDesc(N_.ELFEL_HEAT, 3, N_.ptr(pc), N_.ptr(w), nn, sp, N_.Space())
    am0 = E.start(E.SysmatAssemblerGPU(), nn, nn)
    lib, h = am0._hd.lib, am0._hd.h
    am0._hd.check(lib.elfel_fused_setup(h, ctypes.byref(d)))
    am0._hd.check(lib.elfel_fused_heat(h, None, -6.0))
    K = am0._hd.csc()
    F = np.ones(nn)
    am0._hd.check(lib.elfel_sysmat_rhs(h, N_.ptr(F)))
    assert K.shape == (nn, nn) and K.nnz == 0 and (F == 0.0).all()


def _csc_pinned(E, hd):
    """elfel_sysmat_csc into pinned host arrays (1-based colptr, rowval, values)."""
    import ctypes
    torch = pytest.importorskip("torch")
    N_ = E._native
    nr, nc, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    hd.check(hd.lib.elfel_sysmat_dims(hd.h, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(nnz)))
    cp = torch.full((nc.value + 1,), -7, dtype=torch.int64).pin_memory()
    rv = torch.full((max(nnz.value, 1),), -7, dtype=torch.int64).pin_memory()
    nz = torch.full((max(nnz.value, 1),), np.nan, dtype=torch.float64).pin_memory()

    def p(t, typ):
        return ctypes.cast(ctypes.c_void_p(t.data_ptr()), typ)

    hd.check(hd.lib.elfel_sysmat_csc(hd.h, p(cp, N_._i64p), p(rv, N_._i64p), p(nz, N_._dp)))
    k = nnz.value
    return cp.numpy().copy(), rv.numpy()[:k].copy(), nz.numpy()[:k].copy()


def test_csc_pinned_output(E, O, gpu):
    """CSC output into pinned arrays: the indices are written by a kernel on the
    auxiliary stream from the moment the pattern is complete, alongside an
    assembly still running on the context stream; the values are copied after
    it.  Equal to the staged copy into pageable arrays, right after a fused
    assembly (first and tile form) and after a COO assembly."""
    mesh = E.jitter(E.T6block(1.0, 1.0, 90, 70), 0.1 / 90, seed=2)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    n = E.ndofs(fesp)
    kappa = np.exp(np.random.default_rng(1).uniform(np.log(0.5), np.log(2.0), mesh.nel))
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"kind": "default", "npts": 3}), kappa, -6.0)
    for rep in range(3):
        if rep:
            am.heat(None, -6.0)  # not awaited: the pinned output follows it directly
        cp, rv, nz = _csc_pinned(E, am._hd)
        K = am.csc()
        assert np.array_equal(cp, K.indptr + 1) and np.array_equal(rv, K.indices + 1)
        assert np.array_equal(nz.view(np.int64), K.data.view(np.int64)), rep
    rng = np.random.default_rng(3)
    I, J = rng.integers(1, 301, 50000), rng.integers(1, 201, 50000)
    V = rng.standard_normal(50000)
    a = E.start(E.SysmatAssemblerSparse(0.0), 300, 200)
    a._chunks.append((I, J, V))
    A = E.finish(a)
    cp, rv, nz = _csc_pinned(E, a._hd)
    assert np.array_equal(cp, A.indptr + 1) and np.array_equal(rv, A.indices + 1)
    assert np.array_equal(nz, A.data)
