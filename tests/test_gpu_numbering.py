"""DOF numbering and element DOF tables built on the device.

numberdofs! of one space or of several (src/FESpaces.jl:250-259,
src/FEFields.jl:137-177) runs as exclusive scans over the essential-BC masks
on the device (elfel_number_dofs), and the fused set-up can build the
FEIterator DOF tables from the connectivity (elfel_fused_setup_numbered).  The
numbers must equal the host mirror's (fespaces.py) bit for bit -- on the
reference's own fixtures (qmesh with its EBC nodes, scalar and 3-component;
mt3gen3 with the EBCs of test/test_fefields.jl), on partial essential-BC sets,
on the Taylor-Hood pair and on spaces without free or without data DOFs -- and
the assembled K must be the same bits as with the host-built tables.
"""
import numpy as np
import pytest

from problems import elasticity_setup, stokes_setup

pytestmark = pytest.mark.gpu


def _host_then_device(E, spaces):
    """(host numbers, device numbers, host nunknowns, device nunknowns)."""
    E.numberdofs(spaces if len(spaces) > 1 else spaces[0])
    host = [sp.field.dofnums.copy() for sp in spaces]
    nu_host = sum(E.nunknowns(sp) for sp in spaces)
    for sp in spaces:
        sp.field.dofnums[:] = 0
    nu_dev = E.numberdofs_device(spaces if len(spaces) > 1 else spaces[0])
    dev = [sp.field.dofnums.copy() for sp in spaces]
    return host, dev, nu_host, nu_dev


def _same_bits(K1, K2):
    return (np.array_equal(K1.indptr, K2.indptr) and np.array_equal(K1.indices, K2.indices)
            and np.array_equal(K1.data.view(np.int64), K2.data.view(np.int64)))


def test_qmesh_numbering_golden(E, gpu, golden):
    """test/test_feiterators.jl:21-71, 140-172: qmesh with its EBC nodes, 1 and 3 components."""
    g = golden("feiterators.json")
    mesh = E.T3block(1.0, 1.0, 2, 3)
    fesp = E.FESpace(float, mesh, E.FEH1_T3())
    E.setebc(fesp, 0, np.array(g["ebc_nodes"]), 1, 0.0)
    host, dev, nh, nd = _host_then_device(E, [fesp])
    assert np.array_equal(dev[0], host[0]) and nd == nh == g["scalar_nunknowns_ebc"]
    assert dev[0][:, 0].tolist() == g["scalar_dofnum_by_node"]
    f3 = E.FESpace(float, mesh, E.FEH1_T3(), 3)
    for i in g["ebc_nodes"]:
        E.setebc(f3, 0, i, 1, 0.0)
    host, dev, nh, nd = _host_then_device(E, [f3])
    assert np.array_equal(dev[0], host[0]) and nd == nh
    assert E.FEIterator(f3).eldofs_table().tolist() == g["vec3_eldofs"]


def test_mt3gen3_numbering_golden(E, gpu, golden):
    """test/test_fefields.jl:13-52: 2 DOFs per term, two EBCs."""
    gm, g = golden("meshes.json"), golden("fefields.json")
    mesh = E.Mesh("T3", np.array(gm["mt3gen3_conn"]), np.array(gm["mt3gen3_xyz"])[:, :2])
    fesp = E.FESpace(float, mesh, E.FEH1_T3(), 2)
    for tid, comp, val in g["ebc"]:
        E.setebc(fesp, 0, tid, comp, val)
    host, dev, nh, nd = _host_then_device(E, [fesp])
    assert np.array_equal(dev[0], host[0]) and nd == nh
    f = fesp.field
    assert f.highestfreedofnum() == g["highest_free_ebc"] and f.highestdatadofnum() == g["highest_data_ebc"]


@pytest.mark.parametrize("case", ["cavity", "no_velocity_data", "no_free", "three_spaces"])
def test_several_spaces(E, gpu, case):
    """numberdofs!([fesp1, fesp2, ...]): the Taylor-Hood pair of the cavity, and
    the chaining of first numbers when a space has no data or no free DOFs."""
    rng = np.random.default_rng(3)
    if case == "cavity":
        vmesh, pmesh, uf, pf = stokes_setup(E, 8, lid=True)
        spaces = [uf, pf]
    else:
        vmesh = E.T6block(1.0, 1.0, 5, 4)
        pmesh = E.T6toT3(vmesh)
        uf = E.FESpace(float, vmesh, E.FEH1_T6(), 2)
        pf = E.FESpace(float, pmesh, E.FEH1_T3(), 1)
        spaces = [uf, pf]
        if case == "no_velocity_data":
            E.setebc(pf, 0, 1, 1, 0.0)
        elif case == "no_free":
            E.setebc(uf, 0, np.arange(1, vmesh.nnodes + 1), 1, 0.0)
            E.setebc(uf, 0, np.arange(1, vmesh.nnodes + 1), 2, 0.0)
            E.setebc(pf, 0, rng.choice(pmesh.nnodes, 5, replace=False) + 1, 1, 0.0)
        else:
            tf = E.FESpace(float, vmesh, E.FEH1_T6(), 3)
            for comp in (1, 2, 3):
                E.setebc(tf, 0, rng.choice(vmesh.nnodes, 7, replace=False) + 1, comp, 0.0)
            E.setebc(uf, 0, rng.choice(vmesh.nnodes, 9, replace=False) + 1, 1, 0.0)
            spaces = [uf, pf, tf]
    host, dev, nh, nd = _host_then_device(E, spaces)
    for h, d in zip(host, dev):
        assert np.array_equal(h, d), case
    assert nh == nd


def test_fused_numbered_heat_partial_ebc(E, gpu):
    """T6 heat with only the left and bottom edges fixed: numbers and K from the
    device tables equal those from the host tables, bit for bit."""
    mesh = E.jitter(E.T6block(1.0, 1.0, 23, 17), 0.01, seed=4)
    kappa = np.linspace(0.5, 2.0, mesh.nel)
    xy = mesh.xy
    fixed = np.nonzero((np.abs(xy[:, 0]) < 1e-12) | (np.abs(xy[:, 1]) < 1e-12))[0] + 1

    def space():
        f = E.FESpace(float, mesh, E.FEH1_T6())
        E.setebc(f, 0, fixed, 1, 1.0 + xy[fixed - 1, 0] ** 2)
        return f

    f1 = space()
    E.numberdofs(f1)
    n = E.ndofs(f1)
    qp = E.QPIterator(f1, {"npts": 3})
    am1 = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am1, E.FEIterator(f1), qp, kappa, -6.0)
    f2 = space()
    am2 = E.start(E.SysmatAssemblerGPU(), n, n)
    nu = am2.setup_numbered(1, f2, qp)
    am2.heat(kappa, -6.0)
    assert np.array_equal(f2.field.dofnums, f1.field.dofnums) and nu == E.nunknowns(f1)
    assert _same_bits(E.finish(am1), E.finish(am2))
    assert np.array_equal(am1.rhs().view(np.int64), am2.rhs().view(np.int64))
    _, _, dofs = am2.tables()
    assert np.array_equal(dofs, E.FEIterator(f1).eldofs_table())


def test_fused_numbered_elasticity_and_stokes(E, gpu):
    mesh, fesp, bforce, right = elasticity_setup(E, 12, 6)
    n = E.ndofs(fesp)
    qp = E.QPIterator(fesp, {"npts": 3})
    am1 = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_elasticity(am1, E.FEIterator(fesp), qp, 1.0, 0.3, True, bforce, right, (1.0, 0.0))
    ref = fesp.field.dofnums.copy()
    fesp.field.dofnums[:] = 0
    am2 = E.start(E.SysmatAssemblerGPU(), n, n)
    am2.setup_numbered(2, fesp, qp)
    am2.elasticity(1.0, 0.3, True, bforce, right, (1.0, 0.0))
    assert np.array_equal(fesp.field.dofnums, ref)
    assert _same_bits(E.finish(am1), E.finish(am2))

    vmesh, pmesh, uf, pf = stokes_setup(E, 9, lid=True)
    n = E.ndofs(uf) + E.ndofs(pf)
    qp = E.QPIterator(uf, {"npts": 3})
    am1 = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_stokes(am1, E.FEIterator(uf), E.FEIterator(pf), qp, 1.0)
    refs = [uf.field.dofnums.copy(), pf.field.dofnums.copy()]
    uf.field.dofnums[:] = 0
    pf.field.dofnums[:] = 0
    am2 = E.start(E.SysmatAssemblerGPU(), n, n)
    am2.setup_numbered(3, uf, qp, pf)
    am2.stokes(1.0)
    assert np.array_equal(uf.field.dofnums, refs[0]) and np.array_equal(pf.field.dofnums, refs[1])
    assert _same_bits(E.finish(am1), E.finish(am2))
