"""Host-side mirror of the Elfel.jl API and the C ABI surface (no GPU)."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_t3block_matches_fixture(E, golden):
    """The block generator reproduces the reference's qmesh fixture (3 x 4 nodes)."""
    gm = golden("meshes.json")
    m = E.T3block(1.0, 1.0, 2, 3)
    assert m.conn.tolist() == gm["qmesh_conn"]
    assert np.allclose(m.xy, gm["qmesh_xyz"])


def test_space_numbering_golden(E, golden):
    """test/test_feiterators.jl:21-71, 140-172 through FESpace/FEIterator."""
    g = golden("feiterators.json")
    mesh = E.T3block(1.0, 1.0, 2, 3)
    fesp = E.FESpace(float, mesh, E.FEH1_T3())
    E.numberfreedofs(fesp)
    E.numberdatadofs(fesp)
    assert E.ndofs(fesp) == g["scalar_ndofs"] and E.nunknowns(fesp) == g["scalar_nunknowns_free"]
    E.setebc(fesp, 0, np.array(g["ebc_nodes"]), 1, 0.0)
    E.numberfreedofs(fesp)
    E.numberdatadofs(fesp)
    assert E.nunknowns(fesp) == g["scalar_nunknowns_ebc"]
    it = E.FEIterator(fesp)
    for el in it:
        assert E.eldofs(el).tolist() == [g["scalar_dofnum_by_node"][n - 1] for n in E.elnodes(el)]
    f3 = E.FESpace(float, mesh, E.FEH1_T3(), 3)
    for i in g["ebc_nodes"]:
        E.setebc(f3, 0, i, 1, 0.0)
    E.numberfreedofs(f3)
    E.numberdatadofs(f3)
    it3 = E.FEIterator(f3)
    assert E.eldofcomps(it3).tolist() == g["vec3_eldofcomps"]
    assert it3.eldofs_table().tolist() == g["vec3_eldofs"]
    assert [E.eldofs(el).tolist() for el in E.FEIterator(f3)] == g["vec3_eldofs"]


def test_edof_tables(E):
    """test/test_fespaces.jl:147-167 (edofmdim/edofbfnum/edofcompnt)."""
    f = E.FESpace(float, E.T3block(1.0, 1.0, 2, 3), E.FEH1_T3(), 3)
    assert E.edofmdim(f).tolist() == [0] * 9
    assert E.edofbfnum(f).tolist() == [1, 1, 1, 2, 2, 2, 3, 3, 3]
    assert E.edofcompnt(f).tolist() == [1, 2, 3] * 3
    assert E.dofnum(f, 0, 1, 1) == 0


def test_fefield_mt3gen3(E, golden):
    """test/test_fefields.jl:13-52 through FEField."""
    gm = golden("meshes.json")
    g = golden("fefields.json")
    nt = len(gm["mt3gen3_xyz"])
    f = E.FEField(2, nt)
    f.numberfreedofs()
    f.numberdatadofs(f.freedofnums()[1] + 1)
    assert f.highestfreedofnum() == g["highest_free_no_ebc"] and f.datadofnums()[2] == 0
    for tid, comp, val in g["ebc"]:
        f.setebc(tid, comp, val)
    f.numberfreedofs(1)
    f.numberdatadofs(f.freedofnums()[1] + 1)
    assert f.highestfreedofnum() == g["highest_free_ebc"]
    assert f.highestdatadofnum() == g["highest_data_ebc"]
    v = np.zeros(f.ndofs())
    f.gathersysvec(v)
    assert v[nt * 2 - 2] == 3.0


def test_qpiterator_tables(E, golden):
    g = golden("qpiterators.json")
    fesp = E.FESpace(float, E.T3block(1.0, 1.0, 2, 3), E.FEH1_T3())
    qp1 = E.QPIterator(fesp, {"kind": "default"})
    assert len(qp1) == 1
    for q in qp1:
        assert np.allclose(E.bfun(q), g["t3_1pt_N"][0])
    qp3 = E.QPIterator(fesp, {"kind": "default", "npts": 3})
    assert len(qp3) == 3
    for k, q in enumerate(qp3):
        assert np.allclose(E.bfun(q), g["t3_3pt_N"][k])
        assert np.allclose(E.bfungradpar(q), g["t3_gradpar"])
        assert E.weight(q) == g["weight_3pt"]


def test_local_assembler_append_order(E, O):
    """assemble! appends column-major, assemble!(transpose) row-major and swapped (Assemblers.jl:97-114)."""
    rng = np.random.default_rng(1)
    m = rng.standard_normal((3, 4))
    gi, gj = np.array([1, 7, 5]), np.array([5, 2, 1, 4])
    la = E.LocalMatrixAssembler(3, 4, 0.0)
    E.init(la, gi, gj)
    for j in range(1, 5):
        for i in range(1, 4):
            la[i, j] += m[i - 1, j - 1]
    a = E.start(E.SysmatAssemblerSparse(0.0), 7, 7)
    E.assemble(a, la)
    E.assemble(a, E.transpose(la))
    E.assemble(a, 3, 6, 0.5)
    I, J, V = a.triplets()
    ke = m.ravel(order="F")[None, :]
    I1, J1, V1 = O.local_coo(gi[None, :] - 1, gj[None, :] - 1, ke)
    I2, J2, V2 = O.local_coo_transpose(gi[None, :] - 1, gj[None, :] - 1, ke)
    assert (I - 1).tolist() == I1.tolist() + I2.tolist() + [2]
    assert (J - 1).tolist() == J1.tolist() + J2.tolist() + [5]
    assert V.tolist() == V1.tolist() + V2.tolist() + [0.5]


def test_t6_mesh_and_t6tot3(E):
    m = E.T6block(2.0, 1.0, 4, 3)
    assert m.nel == 24 and m.nnodes == 9 * 7
    x, y = m.xy[:, 0], m.xy[:, 1]
    c = m.conn - 1
    for k in range(3):  # midside k+3 is the midpoint of edge (k, k+1)
        a, b, mid = c[:, k], c[:, (k + 1) % 3], c[:, 3 + k]
        assert (x[mid] == 0.5 * (x[a] + x[b])).all() and (y[mid] == 0.5 * (y[a] + y[b])).all()
    # counter-clockwise elements
    det = (x[c[:, 1]] - x[c[:, 0]]) * (y[c[:, 2]] - y[c[:, 0]]) - (y[c[:, 1]] - y[c[:, 0]]) * (x[c[:, 2]] - x[c[:, 0]])
    assert (det > 0).all()
    p = E.T6toT3(m)
    assert p.nnodes == 5 * 4 and p.nel == 24
    assert np.allclose(p.xy, m.xy[p.vertex_nodes - 1])
    j = E.jitter(m, 0.05, seed=1)
    jc = E.jitter(m, 0.05, seed=1, curved=True)
    assert (j.xy[E.boundary_nodes(m) - 1] == m.xy[E.boundary_nodes(m) - 1]).all()
    for k in range(3):
        a, b, mid = c[:, k], c[:, (k + 1) % 3], c[:, 3 + k]
        assert (j.xy[mid] == 0.5 * (j.xy[a] + j.xy[b])).all()
    assert not np.allclose(jc.xy, j.xy)


def test_alternate_orientation_counts(E):
    m = E.T3block(1.0, 1.0, 4, 4, orientation="alternate")
    assert m.nel == 32
    # interior vertex valence alternates 4 / 8
    val = np.bincount(m.conn.ravel() - 1, minlength=m.nnodes)
    assert sorted(set(val[[6, 7, 8, 11, 12, 13, 16, 17, 18]].tolist())) == [4, 8]


def _header_symbols():
    with open(os.path.join(ROOT, "include", "elfel_gpu.h")) as f:
        h = f.read()
    return sorted(set(re.findall(r"ELFEL_API\s+[\w\s\*]+?\b(elfel_\w+)\s*\(", h)))


def test_library_exports_header_symbols(E):
    """libelfel_gpu.so loads and exports every function include/elfel_gpu.h declares."""
    E.build()
    lib = ctypes.CDLL(E._native.LIB_PATH)
    syms = _header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(E._native.SIGNATURES)
    lib.elfel_abi_version.restype = ctypes.c_int
    assert lib.elfel_abi_version() == 2


def test_no_cpu_fallback_without_library(E, tmp_path):
    """The product path raises when the library is missing; nothing runs on the CPU instead."""
    import pytest

    with pytest.raises(ImportError):
        E._native.load(str(tmp_path / "missing.so"))
