"""The exact-rational T6 heat record, checked on the oracle's element matrices (CPU).

For a straight-sided T6 element (midside nodes at the edge midpoints) and a
quadrature rule exact for the gradient products (the 3-point rule), the 21
stored entries of the element conductivity matrix (column-packed upper
triangle, s = j (j + 1) / 2 + i) take only the values b0..b5 (entries 0..5),
b6 (entry 9), -4 or -8 times b1, b3 or b4, or zero, and the element load is
zero at the vertices and equal at the three midside nodes.  The device's T6
kernels and the tile reduction rely on this (t6r.cuh: kT6REntry, t6r_entry,
t6r_table).  Checked here on the oracle's quadrature-loop matrices
(test/test_heat.jl:49-54) for random elements, within 1e-13 of the largest
entry, and the packed 4-bit form of the map against its table.
"""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _entry_table():
    src = open(os.path.join(ROOT, "elfel.jl_gb300", "csrc", "t6r.cuh")).read()
    m = re.search(r"kT6REntry\[21\]\s*=\s*\{([^}]*)\}", src)
    table = [int(x) for x in m.group(1).split(",")]
    words = re.search(r"0x([0-9a-f]+)ull >> \(4 \* s\)\).*?0x([0-9a-f]+)u >> \(4 \* \(s - 16\)\)", src, re.S)
    lo, hi = int(words.group(1), 16), int(words.group(2), 16)
    packed = [(lo >> (4 * s)) & 15 if s < 16 else (hi >> (4 * (s - 16))) & 15 for s in range(21)]
    return table, packed


def test_packed_entry_map_matches_table():
    table, packed = _entry_table()
    assert len(table) == 21 and packed == table
    assert set(table) <= set(range(14))


def _random_t6(rng, E):
    """E straight-sided T6 elements (positively oriented, not degenerate)."""
    xy = []
    for _ in range(E):
        while True:
            p = rng.uniform(-1.0, 1.0, (3, 2)) * rng.uniform(1e-3, 10.0)
            det = (p[1, 0] - p[0, 0]) * (p[2, 1] - p[0, 1]) - (p[2, 0] - p[0, 0]) * (p[1, 1] - p[0, 1])
            if abs(det) > 1e-3 * np.abs(p).max() ** 2:
                break
        if det < 0:
            p = p[[0, 2, 1]]
        m = np.array([(p[0] + p[1]) / 2, (p[1] + p[2]) / 2, (p[2] + p[0]) / 2])
        xy.append(np.vstack([p, m]))
    xy = np.vstack(xy)
    conn0 = np.arange(6 * E, dtype=np.int64).reshape(E, 6)
    return conn0, xy


def test_t6_exact_rational_identity(O):
    rng = np.random.default_rng(31)
    E = 400
    conn0, xy = _random_t6(rng, E)
    kappa = np.exp(rng.uniform(np.log(0.5), np.log(2.0), E))
    ke, fe = O.heat_element_matrices(6, 3, conn0, xy, kappa, -6.0)
    table, _ = _entry_table()
    for e in range(E):
        K = ke[e].reshape(6, 6, order="F")  # column-major, ke[i + 6 j]
        packed = np.array([K[i, j] for j in range(6) for i in range(j + 1)])
        b = [packed[0], packed[1], packed[2], packed[3], packed[4], packed[5], packed[9]]
        v = b + [0.0, -4 * b[1], -4 * b[3], -4 * b[4], -8 * b[1], -8 * b[3], -8 * b[4]]
        tol = 1e-13 * np.abs(packed).max()
        for s in range(21):
            assert abs(packed[s] - v[table[s]]) <= tol, (e, s, packed[s], v[table[s]])
        assert np.allclose(K, K.T, rtol=0, atol=tol)
        f = fe[e]
        ftol = 1e-13 * np.abs(f).max()
        assert np.abs(f[:3]).max() <= ftol and np.ptp(f[3:]) <= ftol, f
