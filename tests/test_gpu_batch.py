"""Batched solves (GPU): many systems iterated in the same launches.

Bars:
  * every batched solve reaches rtol (FP64 residual computed on the device)
    and matches the oracle's direct solve within ERR_TOL (relative, max norm);
  * a system's solution is bit-identical (tolerance 0) alone in a batch and
    in any mix, whenever it joins: the batched arithmetic of one system never
    depends on the others, nor on the grid the autotuner picks.
"""
import numpy as np
import pytest

from problems import heat_oracle, heat_space

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-8

# (element type, N, orientation, jitter, conductivity seed)
MIX = [("T3", 9, "a", 0.0, 1), ("T6", 14, "alternate", 0.2, 2), ("T3", 48, "alternate", 0.1, 3),
       ("T6", 30, "a", 0.0, 4), ("T3", 3, "a", 0.0, 5), ("T6", 41, "a", 0.15, 6)]


def make(E, etype, N, orient, jit, seed):
    blk = E.T3block if etype == "T3" else E.T6block
    mesh = blk(1.0, 1.0, N, N, orientation=orient)
    if jit:
        mesh = E.jitter(mesh, jit / N, seed=seed)
    fesp = heat_space(E, mesh, E.FEH1_T3() if etype == "T3" else E.FEH1_T6())
    n, nu = E.ndofs(fesp), E.nunknowns(fesp)
    kappa = np.exp(np.random.default_rng(seed).uniform(np.log(0.5), np.log(2.0), mesh.nel))
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"npts": 3}), kappa, -6.0)
    T = np.zeros(n)
    E.gathersysvec(T, fesp)
    return dict(mesh=mesh, fesp=fesp, am=am, T=T, nu=nu, kappa=kappa)


def alone(E, p, method, rtol):
    b = E.BatchSolver(method, capacity=2)
    s = b.add(p["am"], p["T"], p["nu"], rtol=rtol)
    out = b.run()
    b.close()
    return out[s]


@pytest.mark.parametrize("method", ["pcg32_ir", "pcg64"])
def test_batch_matches_direct_and_alone(E, O, gpu, method):
    rtol = 1e-10
    probs = [make(E, *m) for m in MIX]
    ref = [alone(E, p, method, rtol) for p in probs]
    b = E.BatchSolver(method, capacity=8)
    slots = [b.add(p["am"], p["T"], p["nu"], rtol=rtol) for p in probs]
    out = b.run(graphs=2)
    b.close()
    for p, s, (Ta, sta) in zip(probs, slots, ref):
        T, st = out[s]
        assert st["converged"] and st["relres"] <= rtol, st
        assert np.array_equal(T, Ta), "batched result differs from the same system alone"
        assert st["iterations"] == sta["iterations"]
        K0, F0 = heat_oracle(E, O, p["mesh"], p["fesp"], 3, p["kappa"], -6.0)
        T0 = O.solve_lifted(K0, F0, p["T"].copy(), p["nu"])
        assert np.abs(T - T0).max() / np.abs(T0).max() < ERR_TOL


def test_batch_staggered_joins_equal_alone(E, gpu):
    """Systems joining while others iterate (continuous batching) get the same bits."""
    probs = [make(E, *m) for m in MIX]
    ref = [alone(E, p, "pcg32_ir", 1e-10)[0] for p in probs]
    b = E.BatchSolver("pcg32_ir", capacity=4)
    pending = list(range(len(probs)))
    slot_of = {}
    got = {}
    while pending or slot_of:
        # admit one system per step while a slot is free
        if pending and len(slot_of) < 4:
            i = pending.pop(0)
            slot_of[b.add(probs[i]["am"], probs[i]["T"], probs[i]["nu"], rtol=1e-10)] = i
        b.step(1)
        for s in b.done():
            got[slot_of.pop(s)] = b.result(s)[0]
    b.close()
    for i in range(len(probs)):
        assert np.array_equal(got[i], ref[i]), f"system {i}"


def test_batch_same_as_single_solve(E, gpu):
    """The batched PCG64 and the one-system PCG64 agree to rounding (different
    reduction trees), and both converge."""
    p = make(E, "T6", 20, "a", 0.1, 7)
    T1 = p["T"].copy()
    st1 = E.solve(T1, p["am"], None, p["nu"], method="pcg64", rtol=1e-11)
    T2, st2 = alone(E, p, "pcg64", 1e-11)
    assert st1["converged"] and st2["converged"]
    assert np.abs(T1 - T2).max() / np.abs(T1).max() < 1e-9


def test_batch_holds_system_and_errors(E, gpu):
    p = make(E, "T3", 6, "a", 0.0, 8)
    b = E.BatchSolver("pcg32_ir", capacity=1)
    b.add(p["am"], p["T"], p["nu"])
    with pytest.raises(E.ElfelError):  # slots full
        b.add(p["am"], p["T"], p["nu"])
    with pytest.raises(E.ElfelError):  # the system is held by the batch
        p["am"].heat(1.0, -6.0)
    out = b.run()
    assert len(out) == 1
    p["am"].heat(1.0, -6.0)  # released with its result
    b.close()
    with pytest.raises(ValueError):
        E.BatchSolver("minres64")


@pytest.mark.parametrize("method", ["pcg32_ir", "pcg64"])
def test_persistent_form_same_bits(E, gpu, method, monkeypatch):
    """The persistent form (one cooperative launch per group of iterations, grid
    barriers between the phases, ELFEL_BATCH_PERSIST=1) iterates exactly as the
    graphs of three kernels: the same solutions bit for bit and the same
    iteration counts."""
    rtol = 1e-10
    probs = [make(E, *m) for m in MIX[:4]]

    def run():
        b = E.BatchSolver(method, capacity=8)
        slots = [b.add(p["am"], p["T"], p["nu"], rtol=rtol) for p in probs]
        out = b.run(graphs=2)
        b.close()
        return [out[s] for s in slots]

    monkeypatch.setenv("ELFEL_BATCH_PERSIST", "0")
    graph_res = run()
    monkeypatch.setenv("ELFEL_BATCH_PERSIST", "1")
    pers_res = run()
    for (Tg, stg), (Tp, stp) in zip(graph_res, pers_res):
        assert stp["converged"] and stp["relres"] <= rtol, stp
        assert np.array_equal(Tg, Tp) and stg["iterations"] == stp["iterations"]
