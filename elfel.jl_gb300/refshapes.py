"""Reference shapes and quadrature rules (mirror of Elfel.jl src/RefShapes.jl).

Shapes: point, interval, square, cube, triangle, tetrahedron
(src/RefShapes.jl:10-52).  Rules: Gauss on the interval and, as a tensor
product, on the square (src/RefShapes.jl:85-112, 301-361); the triangle rules
by number of points (src/RefShapes.jl:113-246); the tetrahedron rules
(src/RefShapes.jl:248-281).  The tabulated points and weights are the
published rules with the decimals the reference uses, so that element
matrices agree to the last bit with a port of the reference.
"""
import numpy as np


class _RefShape:
    manifdim = 0

    def __repr__(self):
        return type(self).__name__


class RefShapePoint(_RefShape):
    """0-manifold (src/RefShapes.jl:16)."""
    manifdim = 0


class RefShapeInterval(_RefShape):
    """1-manifold, parameter in [-1, 1] (src/RefShapes.jl:23)."""
    manifdim = 1


class RefShapeSquare(_RefShape):
    """Logically rectangular 2-manifold, parameters in [-1, 1]^2 (src/RefShapes.jl:31)."""
    manifdim = 2


class RefShapeCube(_RefShape):
    """3-manifold bounded by six quadrilaterals (src/RefShapes.jl:38)."""
    manifdim = 3


class RefShapeTriangle(_RefShape):
    """Logically triangular 2-manifold (src/RefShapes.jl:46-52)."""
    manifdim = 2


class RefShapeTetrahedron(_RefShape):
    """3-manifold bounded by four triangles (src/RefShapes.jl:52)."""
    manifdim = 3


def manifdim(rs):
    return rs.manifdim


class IntegRule:
    """Quadrature rule: npts, param_coords (npts x dim), weights (src/RefShapes.jl:75-83)."""

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


def _golub_welsch(n):
    """n-point Gauss-Legendre rule on [-1, 1] from the eigen-decomposition of
    the Jacobi matrix (Golub and Welsch, 1969): nodes are the eigenvalues,
    weights 2 v_1^2 of the normalised eigenvectors.  Used above order 5 as in
    src/RefShapes.jl:86-90."""
    k = np.arange(1, n, dtype=np.float64)
    off = k / np.sqrt(4.0 * k * k - 1.0)
    T = np.diag(off, 1) + np.diag(off, -1)
    lam, V = np.linalg.eigh(T)
    return lam, 2.0 * V[0, :] ** 2


def _gauss1(order):
    """Gauss points and weights on [-1, 1] by order (src/RefShapes.jl:85-112)."""
    if order == 1:
        return [0.0], [2.0]
    if order == 2:
        return [-0.577350269189626, 0.577350269189626], [1.0, 1.0]
    if order == 3:
        return [-0.774596669241483, 0.0, 0.774596669241483], [0.5555555555555556, 0.8888888888888889,
                                                              0.5555555555555556]
    if order == 4:
        return ([-0.86113631159405, -0.33998104358486, 0.33998104358486, 0.86113631159405],
                [0.34785484513745, 0.65214515486255, 0.65214515486255, 0.34785484513745])
    if order == 5:
        return ([-0.906179845938664, -0.538469310105683, 0.0, 0.538469310105683, 0.906179845938664],
                [0.236926885056189, 0.478628670499367, 0.568888888888889, 0.478628670499367, 0.236926885056189])
    if order < 1:
        raise ValueError(f"Gauss rule of order {order}")
    x, w = _golub_welsch(int(order))
    return list(x), list(w)


def _triangle(n):
    """Triangle rules by number of points (src/RefShapes.jl:113-246)."""
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
    if n == 9:
        a, b = 0.437525248383384, 0.124949503233232
        c, d, e = 0.165409927389841, 0.037477420750088, 0.797112651860071
        w1, w2 = 0.205950504760887 / 2, 0.063691414286223 / 2
        return ([[a, a], [b, a], [a, b], [c, d], [d, c], [e, c], [c, e], [d, e], [e, d]],
                [w1] * 3 + [w2] * 6)
    if n == 12:
        a, b = 0.063089014491502, 0.873821971016996
        c, d = 0.249286745170910, 0.501426509658179
        e, f, g = 0.310352451033785, 0.053145049844816, 0.636502499121399
        w1, w2, w3 = 0.050844906370207 / 2, 0.116786275726379 / 2, 0.082851075618374 / 2
        return ([[a, a], [b, a], [a, b], [c, c], [d, c], [c, d], [e, f], [f, e], [g, e], [e, g], [f, g], [g, f]],
                [w1] * 3 + [w2] * 3 + [w3] * 6)
    if n == 13:
        a, b, c = 0.479308067841923, 0.260345966079038, 0.869739794195568
        d, e, f, g = 0.065130102902216, 0.638444188569809, 0.312865496004875, 0.048690315425316
        w0, w1, w2, w3 = -0.149570044467670 / 2, 0.175615257433204 / 2, 0.053347235608839 / 2, 0.077113760890257 / 2
        return ([[0.333333333333333, 0.333333333333333], [a, b], [b, a], [b, b], [c, d], [d, c], [d, d],
                 [e, f], [e, g], [f, e], [f, g], [g, e], [g, f]],
                [w0] + [w1] * 3 + [w2] * 3 + [w3] * 6)
    raise ValueError(f"Unknown number of integration points {n}")


def _tetrahedron(n):
    """Tetrahedron rules by number of points (src/RefShapes.jl:248-281)."""
    if n == 1:  # exact for linear polynomials
        return [[0.25, 0.25, 0.25]], [1.0 / 6.0]
    if n == 4:  # exact for quadratics
        a, b = 0.13819660, 0.58541020
        w = 0.041666666666666666667
        return [[a, a, a], [b, a, a], [a, b, a], [a, a, b]], [w, w, w, w]
    if n == 5:  # Zienkiewicz #3
        a, b, c = 1.0 / 6.0, 0.25, 0.5
        return [[b, b, b], [c, a, a], [a, c, a], [a, a, c], [a, a, a]], [-0.8 / 6, 0.45 / 6, 0.45 / 6, 0.45 / 6,
                                                                          0.45 / 6]
    raise ValueError(f"Unknown number of integration points {n}")


def _settings(quadraturesettings):
    qs = dict(quadraturesettings or {})
    kind = qs.get("kind", "default")
    if isinstance(kind, str) and kind.startswith(":"):
        kind = kind[1:]
    return qs, kind


def quadrature(rs=RefShapeTriangle, quadraturesettings=None):
    """quadrature(refshape, (kind=..., npts=... | order=...)) of src/RefShapes.jl:283-361.

    ``quadraturesettings`` is a dict such as {"kind": "default", "npts": 3}
    (triangle, tetrahedron) or {"kind": "Gauss", "order": 2} (interval,
    square).  Defaults: one point.
    """
    qs, kind = _settings(quadraturesettings)
    if rs is RefShapeInterval:
        if kind not in ("default", "Gauss"):
            raise ValueError(f"Integration rule {kind} not available")
        pc, w = _gauss1(int(qs.get("order", 1)))
        return IntegRule(len(w), np.reshape(pc, (-1, 1)), w)
    if rs is RefShapeSquare:
        if kind not in ("default", "Gauss"):
            raise ValueError(f"Integration rule {kind} not available")
        order = int(qs.get("order", 1))
        pc, w = _gauss1(order)
        pts = [[pc[i], pc[j]] for i in range(order) for j in range(order)]  # first coordinate outer
        wts = [w[i] * w[j] for i in range(order) for j in range(order)]
        return IntegRule(len(wts), pts, wts)
    if rs is RefShapeTriangle:
        if kind != "default":
            raise ValueError(f"Integration rule {kind} not available")
        pc, w = _triangle(int(qs.get("npts", 1)))
        return IntegRule(len(w), pc, w)
    if rs is RefShapeTetrahedron:
        if kind != "default":
            raise ValueError(f"Integration rule {kind} not available")
        pc, w = _tetrahedron(int(qs.get("npts", 1)))
        return IntegRule(len(w), pc, w)
    raise NotImplementedError(f"no quadrature rule for {rs}")
