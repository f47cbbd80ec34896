"""Scalar H1 triangle elements T3 and T6 (mirror of Elfel.jl src/FElements.jl:225-288).

The basis functions are evaluated on the host only to build QPIterator
tables; the GPU kernels evaluate them from the same formulas.
"""
import numpy as np

from .refshapes import RefShapeTriangle


class FE:
    refshape = RefShapeTriangle
    name = ""
    nodes_per_elem = 0
    _ndofperfeat = (1, 0, 0, 0)
    _nfeatofdim = (0, 0, 0, 0)

    def nfeatofdim(self, m):
        return self._nfeatofdim[m]

    def ndofperfeat(self, m):
        return self._ndofperfeat[m]

    def ndofsperel(self):
        """Number of DOFs of the scalar element (src/FElements.jl:73-80)."""
        return sum(self.nfeatofdim(m) * self.ndofperfeat(m) for m in range(0, self.manifdim() + 1))

    def manifdim(self):
        return 2

    def __repr__(self):
        return f"FEH1_{self.name}()"


class FEH1_T3(FE):
    """3-node linear triangle; DOFs at the vertices."""
    name = "T3"
    nodes_per_elem = 3
    _nfeatofdim = (3, 3, 1, 0)

    def bfun(self, pc):
        r, s = pc[0], pc[1]
        return np.array([1.0 - r - s, r, s])

    def bfungradpar(self, pc):
        return np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])


class FEH1_T6(FE):
    """6-node quadratic triangle: vertices 1-3, then midsides 1-2, 2-3, 3-1."""
    name = "T6"
    nodes_per_elem = 6
    _nfeatofdim = (6, 3, 1, 0)

    def bfun(self, pc):
        r, s = pc[0], pc[1]
        t = 1.0 - r - s
        return np.array([t * (t + t - 1), r * (r + r - 1), s * (s + s - 1), 4 * r * t, 4 * r * s, 4 * s * t])

    def bfungradpar(self, pc):
        r, s = pc[0], pc[1]
        return np.array([[-3 + 4 * r + 4 * s, -3 + 4 * r + 4 * s], [4 * r - 1, 0.0], [0.0, 4 * s - 1],
                         [4 - 8 * r - 4 * s, -4 * r], [4 * s, 4 * r], [-4 * s, 4 - 4 * r - 8 * s]])


def bfun(fe, pc):
    return fe.bfun(pc)


def bfungradpar(fe, pc):
    return fe.bfungradpar(pc)


def refshape(fe):
    return fe.refshape


def ndofsperel(fe):
    return fe.ndofsperel()


def nfeatofdim(fe, m):
    return fe.nfeatofdim(m)


def ndofperfeat(fe, m):
    return fe.ndofperfeat(m)


def Jacobian(J):
    """Surface Jacobian of a 2x2 Jacobian matrix (src/FElements.jl:120-129)."""
    J = np.asarray(J)
    if J.shape == (2, 2):
        return J[0, 0] * J[1, 1] - J[1, 0] * J[0, 1]
    return float(np.linalg.norm(np.cross(J[:, 0], J[:, 1])))


def jacjac(fe, locs, nodes, gradNpar):
    """(J, det J) with J = sum_j x_j (x) gradNpar_j (src/FElements.jl:148-168); nodes 1-based."""
    X = locs[np.asarray(nodes) - 1]
    J = X.T @ np.asarray(gradNpar)
    return J, Jacobian(J)
