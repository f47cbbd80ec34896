"""Reference shapes and triangle quadrature (mirror of Elfel.jl src/RefShapes.jl).

Only the triangle is on the GPU path (T3/T6 elements).
"""
import numpy as np


class RefShapeTriangle:
    """Logically triangular 2-manifold reference shape (src/RefShapes.jl:46-52)."""
    manifdim = 2


def manifdim(rs):
    return rs.manifdim


class IntegRule:
    """Quadrature rule: npts, param_coords (npts x 2), weights (src/RefShapes.jl:75-83)."""

    def __init__(self, npts, param_coords, weights):
        self.npts = int(npts)
        self.param_coords = np.asarray(param_coords, dtype=np.float64).reshape(self.npts, -1)
        self.weights = np.asarray(weights, dtype=np.float64).reshape(self.npts)


def npts(qr):
    return qr.npts


def param_coords(qr):
    return qr.param_coords


def weights(qr):
    return qr.weights


def _triangle(n):
    """Triangle rules by number of points (src/RefShapes.jl:113-160)."""
    if n == 1:  # exact for linear polynomials
        return [[1.0 / 3.0, 1.0 / 3.0]], [1.0 / 2.0]
    if n == 3:  # exact for quadratics
        return [[2.0 / 3, 1.0 / 6], [1.0 / 6, 2.0 / 3], [1.0 / 6, 1.0 / 6]], [1.0 / 3 / 2, 1.0 / 3 / 2, 1.0 / 3 / 2]
    if n == 4:
        return ([[0.333333333333333, 0.333333333333333], [0.200000000000000, 0.200000000000000],
                 [0.600000000000000, 0.200000000000000], [0.200000000000000, 0.600000000000000]],
                [-0.281250000000000, 0.260416666666667, 0.260416666666667, 0.260416666666667])
    if n == 6:  # exact for quartics
        a, b, c, d = 0.816847572980459, 0.091576213509771, 0.108103018168070, 0.445948490915965
        w1, w2 = 0.109951743655322 / 2, 0.223381589678011 / 2
        return [[a, b], [b, a], [b, b], [c, d], [d, c], [d, d]], [w1, w1, w1, w2, w2, w2]
    if n == 7:
        a, b, c, d = 0.101286507323456, 0.797426958353087, 0.470142064105115, 0.059715871789770
        w1, w2 = 0.062969590272414, 0.066197076394253
        return ([[a, a], [b, a], [a, b], [c, c], [d, c], [c, d], [0.333333333333333, 0.333333333333333]],
                [w1, w1, w1, w2, w2, w2, 0.112500000000000])
    raise ValueError(f"Unknown number of integration points {n}")


def quadrature(rs=RefShapeTriangle, quadraturesettings=None):
    """quadrature(RefShapeTriangle, (kind=:default, npts=...)) of src/RefShapes.jl:301-323.

    ``quadraturesettings`` is a dict such as {"kind": "default", "npts": 3};
    the default rule has one point.
    """
    qs = dict(quadraturesettings or {})
    kind = qs.get("kind", "default")
    if rs is not RefShapeTriangle:
        raise NotImplementedError("only the triangle reference shape is provided")
    if kind != "default":
        raise ValueError(f"Integration rule {kind} not available")
    pc, w = _triangle(int(qs.get("npts", 1)))
    return IntegRule(len(w), pc, w)
