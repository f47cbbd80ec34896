"""Scalar finite elements (mirror of Elfel.jl src/FElements.jl).

H1 (nodal) elements: L2, T3, T6, Q4, T3 with a cubic bubble, T4
(src/FElements.jl:199-386).  L2-conforming (cell-interior) elements with one
constant basis function: FEL2_Q4, FEL2_T3, FEL2_T4 (src/FElements.jl:388-470);
they carry no nodal basis and take their geometry from the nodal element of
the same shape (``geometrycarrier``, src/FElements.jl:190-197).

Each element records its shape's feature counts per manifold dimension (the
MeshCore shape descriptor: vertices, edges, faces, cells) and the number of
degrees of freedom per feature of each dimension.  The basis functions are
evaluated on the host to build QPIterator tables; the device kernels evaluate
the same formulas.
"""
import numpy as np

from .refshapes import RefShapeInterval, RefShapeSquare, RefShapeTetrahedron, RefShapeTriangle

# MeshCore shape descriptors: name -> number of features of dimension 0..3
_SHAPES = {
    "L2": (2, 1, 0, 0),
    "T3": (3, 3, 1, 0),
    "T6": (6, 3, 1, 0),
    "Q4": (4, 4, 1, 0),
    "T4": (4, 6, 4, 1),
}


class ShapeDesc:
    """Topological description of the element's cell (name and feature counts)."""

    def __init__(self, name):
        self.name = name
        self.nfeatofdim = _SHAPES[name]

    @property
    def manifdim(self):
        return max(m for m in range(4) if self.nfeatofdim[m] > 0)

    def __repr__(self):
        return f"ShapeDesc({self.name})"


class FE:
    refshape = RefShapeTriangle
    name = ""
    shape = "T3"
    _ndofperfeat = (1, 0, 0, 0)

    def __init__(self):
        self.sd = ShapeDesc(self.shape)

    @property
    def nodes_per_elem(self):
        """Vertices of the element's cell (the base incidence relation's width)."""
        return self.sd.nfeatofdim[0]

    def nfeatofdim(self, m):
        return self.sd.nfeatofdim[m]

    def ndofperfeat(self, m):
        return self._ndofperfeat[m]

    def ndofsperel(self):
        """Number of DOFs of the scalar element (src/FElements.jl:73-80)."""
        return sum(self.nfeatofdim(m) * self.ndofperfeat(m) for m in range(0, self.manifdim() + 1))

    def manifdim(self):
        return self.refshape.manifdim

    def geometrycarrier(self):
        """The element whose nodal basis maps the geometry (src/FElements.jl:190-197)."""
        return self

    def __repr__(self):
        return f"{type(self).__name__}()"

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self))


class FEH1_L2(FE):
    """2-node linear segment (src/FElements.jl:199-222); parameter in [-1, 1]."""
    refshape = RefShapeInterval
    name = shape = "L2"

    def bfun(self, pc):
        x = pc[0]
        return np.array([(1.0 - x) / 2.0, (1.0 + x) / 2.0])

    def bfungradpar(self, pc):
        return np.array([[-1.0 / 2.0], [1.0 / 2.0]])


class FEH1_T3(FE):
    """3-node linear triangle; DOFs at the vertices (src/FElements.jl:225-246)."""
    name = shape = "T3"

    def bfun(self, pc):
        r, s = pc[0], pc[1]
        return np.array([1.0 - r - s, r, s])

    def bfungradpar(self, pc):
        return np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])


class FEH1_T6(FE):
    """6-node quadratic triangle: vertices 1-3, then midsides 1-2, 2-3, 3-1 (src/FElements.jl:248-288)."""
    name = shape = "T6"

    def bfun(self, pc):
        r, s = pc[0], pc[1]
        t = 1.0 - r - s
        return np.array([t * (t + t - 1), r * (r + r - 1), s * (s + s - 1), 4 * r * t, 4 * r * s, 4 * s * t])

    def bfungradpar(self, pc):
        r, s = pc[0], pc[1]
        return np.array([[-3 + 4 * r + 4 * s, -3 + 4 * r + 4 * s], [4 * r - 1, 0.0], [0.0, 4 * s - 1],
                         [4 - 8 * r - 4 * s, -4 * r], [4 * s, 4 * r], [-4 * s, 4 - 4 * r - 8 * s]])


class FEH1_Q4(FE):
    """4-node bilinear quadrilateral on [-1, 1]^2, counter-clockwise vertices (src/FElements.jl:290-320)."""
    refshape = RefShapeSquare
    name = shape = "Q4"

    def bfun(self, pc):
        x, y = pc[0], pc[1]
        return np.array([0.25 * (1.0 - x) * (1.0 - y), 0.25 * (1.0 + x) * (1.0 - y), 0.25 * (1.0 + x) * (1.0 + y),
                         0.25 * (1.0 - x) * (1.0 + y)])

    def bfungradpar(self, pc):
        x, y = pc[0], pc[1]
        return np.array([[-(1.0 - y) * 0.25, -(1.0 - x) * 0.25], [(1.0 - y) * 0.25, -(1.0 + x) * 0.25],
                         [(1.0 + y) * 0.25, (1.0 + x) * 0.25], [-(1.0 + y) * 0.25, (1.0 - x) * 0.25]])


class FEH1_T3_BUBBLE(FE):
    """Linear triangle plus the cubic interior bubble (1-r-s) r s, one DOF on
    the cell (src/FElements.jl:322-355).  Its own geometry carrier: the
    Jacobian uses the three vertex functions only."""
    name = "T3_BUBBLE"
    shape = "T3"
    _ndofperfeat = (1, 0, 1, 0)

    def bfun(self, pc):
        xi, eta = pc[0], pc[1]
        return np.array([1.0 - xi - eta, xi, eta, (1.0 - xi - eta) * xi * eta])

    def bfungradpar(self, pc):
        xi, eta = pc[0], pc[1]
        return np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0],
                         [-xi * eta + (1.0 - xi - eta) * eta, -xi * eta + (1.0 - xi - eta) * xi]])


class FEH1_T4(FE):
    """4-node linear tetrahedron (src/FElements.jl:357-386)."""
    refshape = RefShapeTetrahedron
    name = shape = "T4"

    def bfun(self, pc):
        r, s, t = pc[0], pc[1], pc[2]
        return np.array([1.0 - r - s - t, r, s, t])

    def bfungradpar(self, pc):
        return np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


class _FEL2(FE):
    """One constant basis function on the cell; geometry from the nodal element."""
    _carrier = FEH1_T3

    def bfun(self, pc):
        return np.array([1.0])

    def bfungradpar(self, pc):
        return np.zeros((1, self.refshape.manifdim))

    def geometrycarrier(self):
        return self._carrier()


class FEL2_Q4(_FEL2):
    """Cell-constant element on quadrilaterals (src/FElements.jl:388-418)."""
    refshape = RefShapeSquare
    name = "L2_Q4"
    shape = "Q4"
    _ndofperfeat = (0, 0, 1, 0)
    _carrier = FEH1_Q4


class FEL2_T3(_FEL2):
    """Cell-constant element on triangles (src/FElements.jl:420-444)."""
    name = "L2_T3"
    shape = "T3"
    _ndofperfeat = (0, 0, 1, 0)
    _carrier = FEH1_T3


class FEL2_T4(_FEL2):
    """Cell-constant element on tetrahedra (src/FElements.jl:446-470)."""
    refshape = RefShapeTetrahedron
    name = "L2_T4"
    shape = "T4"
    _ndofperfeat = (0, 0, 0, 1)
    _carrier = FEH1_T4


def bfun(fe, pc):
    return fe.bfun(pc)


def bfungradpar(fe, pc):
    return fe.bfungradpar(pc)


def refshape(fe):
    return fe.refshape


def shapedesc(fe):
    return fe.sd


def manifdim(fe):
    return fe.manifdim()


def ndofsperel(fe):
    return fe.ndofsperel()


def nfeatofdim(fe, m):
    return fe.nfeatofdim(m)


def ndofperfeat(fe, m):
    return fe.ndofperfeat(m)


def Jacobian(J):
    """Jacobian of the map from the parametric manifold (src/FElements.jl:92-147).

    ``J`` is sdim x mdim: 1 for a point, the length of the tangent for a
    curve, the determinant (square J) or the area of the parallelogram for a
    surface, the determinant for a volume.
    """
    J = np.atleast_2d(np.asarray(J, dtype=np.float64))
    sdim, ntan = J.shape
    if ntan == 0:
        return 1.0
    if ntan == 1:
        return float(np.linalg.norm(J[:, 0]))
    if ntan == 2:
        if sdim == 2:
            return J[0, 0] * J[1, 1] - J[1, 0] * J[0, 1]
        return float(np.linalg.norm(np.cross(J[:, 0], J[:, 1])))
    if ntan == 3 and sdim == 3:
        return (J[0, 0] * (J[1, 1] * J[2, 2] - J[2, 1] * J[1, 2]) - J[0, 1] * (J[1, 0] * J[2, 2] - J[1, 2] * J[2, 0]) +
                J[0, 2] * (J[1, 0] * J[2, 1] - J[1, 1] * J[2, 0]))
    raise ValueError(f"Jacobian of a {sdim} x {ntan} matrix")


def jacjac(fe, locs, nodes, gradNpar):
    """(J, Jacobian) with J = sum_j x_j (x) gradNpar_j over the element's nodes
    (src/FElements.jl:148-168); nodes 1-based.  Only the first len(nodes)
    gradients are used (the bubble's cell function does not map geometry)."""
    nodes = np.asarray(nodes)
    X = np.atleast_2d(np.asarray(locs)[nodes - 1])  # nn x sdim
    G = np.asarray(gradNpar)[: len(nodes)]
    J = X.T @ G
    return J, Jacobian(J)
