"""Device error integrals (GPU): evaluate_pressure_error / evaluate_velocity_error
of Elfel.jl test/test_stokes.jl:438-496 computed on the device.

Bars: the reference's own error norms of the vector-Laplacian Taylor-Hood test
(test/test_stokes.jl:777-780, golden vectors) within 1e-7 relative (the bar of
the host-side check of the same solve), and the oracle's integrals of the same
solution vector within 1e-12 relative (only the summation order differs).
"""
import numpy as np
import pytest

from problems import heat_space, stokes_errors, stokes_setup

pytestmark = pytest.mark.gpu

UX = {(1, 3): 20.0}                      # 20 x y^3
UY = {(4, 0): 5.0, (0, 4): -5.0}         # 5 x^4 - 5 y^4
P = {(2, 1): 60.0, (0, 3): -20.0}        # 60 x^2 y - 20 y^3


def test_stokes_errors_golden(E, O, gpu, golden):
    g = golden("stokes.json")["veclap_th_errors"]
    vmesh, pmesh, ufesp, pfesp = stokes_setup(E, g["N"])
    n = E.ndofs(ufesp) + E.ndofs(pfesp)
    nu = E.nunknowns(ufesp) + E.nunknowns(pfesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_stokes(am, E.FEIterator(ufesp), E.FEIterator(pfesp), E.QPIterator(ufesp, {"npts": 3}), 1.0)
    U = np.zeros(n)
    E.gathersysvec(U, [ufesp, pfesp])
    st = E.solve(U, am, None, nu, method="minres64", rtol=1e-12, maxit=20000)
    assert st["converged"]
    ep = am.error_l2(U, P, space=1)
    ev = am.error_l2(U, [UX, UY], space=0)
    assert np.allclose([ep, ev], g["ep_ev"], rtol=1e-7)
    ep0, ev0 = stokes_errors(O, vmesh, pmesh, ufesp, pfesp, U)
    assert abs(ep - ep0) <= 1e-12 * ep0 and abs(ev - ev0) <= 1e-12 * ev0


@pytest.mark.parametrize("etype", ["T3", "T6"])
def test_heat_error_vs_oracle(E, O, gpu, etype):
    """T = 1 + x^2 + 2 y^2: nodally exact for T3 on uniform diagonals, exact for T6."""
    mesh = (E.T3block if etype == "T3" else E.T6block)(1.0, 1.0, 12, 9)
    fesp = heat_space(E, mesh, E.FEH1_T3() if etype == "T3" else E.FEH1_T6())
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), 1.0, -6.0)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    E.solve(T, am, None, nu, method="pcg64", rtol=1e-12)
    exact = {(0, 0): 1.0, (2, 0): 1.0, (0, 2): 2.0}
    err = am.error_l2(T, exact)
    vals = T[fesp.field.dofnums[:, 0] - 1]
    err0 = O.l2_error_scalar(mesh.conn - 1, mesh.xy, mesh.nodes_per_elem, vals,
                             lambda x, y: 1.0 + x ** 2 + 2.0 * y ** 2)
    # relative 1e-12, or absolute 1e-12 where the error itself is round-off (T6)
    assert abs(err - err0) <= 1e-12 * err0 + 1e-12
    if etype == "T6":
        assert err < 1e-9  # the quadratic is in the T6 space
