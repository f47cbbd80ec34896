"""The tile reduction of resident T6 heat patterns against the contributor-list reduction.

The first assembly of a fused T6 heat system reduces element records through
the pattern's contributor lists (reduce_k); from the second assembly on, an
exact-rule straight-sided mesh writes 8 bases per element and the tile
reduction expands and sums them (tiles.cu).  Both add every nonzero's
contributions in slot order, so K must come out bit for bit the same
(tolerance: none).  The meshes cover deduplicated tile programs (block
meshes), tiles whose programs are all distinct (element order shuffled),
tiles split for their element count, and tiles beyond the limits (a vertex
shared by 20 elements: a nonzero with 20 contributions).
"""
import numpy as np
import pytest

from problems import heat_oracle, heat_space

pytestmark = pytest.mark.gpu


def _fan_t6(m=20):
    """m T6 triangles around a centre vertex (a regular polygon fan)."""
    ang = 2 * np.pi * np.arange(m) / m
    rim = np.stack([np.cos(ang), np.sin(ang)], axis=1)
    xy = [np.zeros(2)] + list(rim)  # node 1: centre, nodes 2..m+1: rim
    conn = []
    spoke = {}
    for k in range(m):
        a, b = 2 + k, 2 + (k + 1) % m
        for v in (a, b):
            if v not in spoke:
                xy.append(0.5 * (xy[0] + xy[v - 1]))
                spoke[v] = len(xy)
        xy.append(0.5 * (xy[a - 1] + xy[b - 1]))
        rim_mid = len(xy)
        conn.append([1, a, b, spoke[a], rim_mid, spoke[b]])
    return np.array(conn), np.array(xy)


def _assemble_twice(E, mesh, fesp, kappa):
    n = E.ndofs(fesp)
    am = E.start(E.SysmatAssemblerGPU(), n, n)
    E.assemble_heat(am, E.FEIterator(fesp), E.QPIterator(fesp, {"kind": "default", "npts": 3}), kappa, -6.0)
    K1, F1 = E.finish(am), am.rhs().copy()
    assert am.tile_stats() == (0, 0, 0, 0)
    am.heat(None, -6.0)
    K2, F2 = E.finish(am), am.rhs().copy()
    am.heat(None, -6.0)
    K3 = E.finish(am)
    return am, (K1, F1), (K2, F2), K3


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


CASES = [
    # name, nx, ny, orientation, jitter, shuffle
    ("block", 40, 30, "a", 0.0, False),
    ("wide", 400, 8, "a", 0.1, False),
    ("jittered", 64, 48, "a", 0.2, False),
    ("alternate", 50, 50, "alternate", 0.1, False),
    ("shuffled", 40, 40, "a", 0.1, True),
    ("tall", 3, 300, "a", 0.1, False),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_tile_reduction_bits(E, O, gpu, case):
    name, nx, ny, orient, jit, shuffle = case
    mesh = E.T6block(1.0, 1.0, nx, ny, orientation=orient)
    if jit:
        mesh = E.jitter(mesh, jit / max(nx, ny), seed=21)
    if shuffle:
        perm = np.random.default_rng(5).permutation(mesh.nel)
        mesh = E.Mesh("T6", mesh.conn[perm], mesh.xy)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    kappa = np.exp(np.random.default_rng(8).uniform(np.log(0.5), np.log(2.0), mesh.nel))
    am, (K1, F1), (K2, F2), K3 = _assemble_twice(E, mesh, fesp, kappa)
    ntiles, nprog, nfb, nruns = am.tile_stats()
    assert ntiles > 0 and nfb == 0 and 0 < nruns <= ntiles
    if name == "wide":
        assert 2 * nprog < ntiles  # translated tiles along the grid lines share their programs
    for K in (K2, K3):
        assert np.array_equal(K.indptr, K1.indptr) and np.array_equal(K.indices, K1.indices)
        assert np.array_equal(_bits(K.data), _bits(K1.data)), name
    assert np.array_equal(_bits(F2), _bits(F1))
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, kappa, -6.0)
    assert np.abs(K2.data - K0.data).max() <= 1e-12 * np.abs(K0.data).max()


def test_tile_reduction_beyond_limits(E, O, gpu):
    """A vertex of 20 elements: its diagonal has 20 contributions, more than a
    tile program holds; that tile is summed from the contributor lists."""
    conn, xy = _fan_t6(20)
    mesh = E.Mesh("T6", conn, xy)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    kappa = np.linspace(0.5, 2.0, mesh.nel)
    am, (K1, F1), (K2, F2), K3 = _assemble_twice(E, mesh, fesp, kappa)
    ntiles, nprog, nfb, nruns = am.tile_stats()
    assert nfb >= 1
    assert np.array_equal(_bits(K2.data), _bits(K1.data))
    assert np.array_equal(_bits(K3.data), _bits(K1.data))
    K0, F0 = heat_oracle(E, O, mesh, fesp, 3, kappa, -6.0)
    assert np.abs(K2.data - K0.data).max() <= 1e-12 * np.abs(K0.data).max()


@pytest.mark.parametrize("run", ["0", "1", "3", "64"])
@pytest.mark.parametrize("case", [CASES[1], CASES[4]], ids=["wide", "shuffled"])
def test_tile_run_lengths_same_bits(E, O, gpu, monkeypatch, run, case):
    """The run kernel (one CTA per run of consecutive tiles of one program,
    the next tile's bases loaded during the current tile's adds) at several
    run lengths, and the one-CTA-per-tile kernel (ELFEL_TILE_RUN=0), give the
    contributor-list values bit for bit."""
    monkeypatch.setenv("ELFEL_TILE_RUN", run)
    name, nx, ny, orient, jit, shuffle = case
    mesh = E.jitter(E.T6block(1.0, 1.0, nx, ny, orientation=orient), jit / max(nx, ny), seed=3)
    if shuffle:
        perm = np.random.default_rng(9).permutation(mesh.nel)
        mesh = E.Mesh("T6", mesh.conn[perm], mesh.xy)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    kappa = np.exp(np.random.default_rng(4).uniform(np.log(0.5), np.log(2.0), mesh.nel))
    am, (K1, F1), (K2, F2), K3 = _assemble_twice(E, mesh, fesp, kappa)
    ntiles, nprog, nfb, nruns = am.tile_stats()
    if run == "0":
        assert nruns == 0
    else:
        assert -(-ntiles // int(run)) <= nruns <= ntiles
        if name == "wide" and run != "1":
            assert nruns < ntiles  # consecutive translated tiles share a run
    for K in (K2, K3):
        assert np.array_equal(_bits(K.data), _bits(K1.data)), (name, run)
    assert np.array_equal(_bits(F2), _bits(F1))


def test_tile_run_beyond_limits(E, O, gpu, monkeypatch):
    """Runs of tiles beyond the limits take the contributor lists in the run kernel."""
    monkeypatch.setenv("ELFEL_TILE_RUN", "4")
    conn, xy = _fan_t6(20)
    mesh = E.Mesh("T6", conn, xy)
    fesp = heat_space(E, mesh, E.FEH1_T6())
    kappa = np.linspace(0.5, 2.0, mesh.nel)
    am, (K1, F1), (K2, F2), K3 = _assemble_twice(E, mesh, fesp, kappa)
    ntiles, nprog, nfb, nruns = am.tile_stats()
    assert nfb >= 1 and nruns >= 1
    assert np.array_equal(_bits(K2.data), _bits(K1.data))
    assert np.array_equal(_bits(K3.data), _bits(K1.data))

