"""Element and quadrature-point iterators.

Mirror of Elfel.jl src/FEIterators.jl and src/QPIterators.jl.  Besides the
per-element iteration of the reference (used by user-written weak forms in
COO mode), FEIterator exposes the whole element DOF table at once
(``eldofs_table``), which is what the fused device assembly consumes.
"""
import numpy as np

from .fespaces import FESpace, edofbfnum, edofcompnt, edofmdim
from .refshapes import quadrature


class FEIterator:
    """Iterates the elements of a space; caches nodes and DOF numbers (src/FEIterators.jl:34-82)."""

    def __init__(self, fesp: FESpace):
        self.fesp = fesp
        self._conn = fesp.mesh.conn
        self._geom = fesp.mesh.xy
        self._state = 0
        self._nodes = np.zeros(fesp.fe.nodes_per_elem, dtype=np.int64)
        self._dofs = np.zeros(fesp.ndofsperel(), dtype=np.int64)
        self._entmdim = np.zeros(fesp.ndofsperel(), dtype=np.int64)  # all DOFs on vertices
        self._dofcomp = np.tile(np.arange(1, fesp.nfecopies + 1), fesp.fe.nodes_per_elem)

    def __len__(self):
        return self._conn.shape[0]

    def __iter__(self):
        for e in range(len(self)):
            self._update(e + 1)
            yield self

    def _update(self, state):
        """Cache the element's nodes and DOFs (src/FEIterators.jl:161-194)."""
        self._state = state
        self._nodes[:] = self._conn[state - 1]
        self._dofs[:] = self.fesp.field.dofnums[self._nodes - 1].ravel()
        return self

    def eldofs_table(self):
        """All elements' DOF numbers (nel x ndofsperel, 1-based), node-major / component-minor."""
        d = self.fesp.field.dofnums[self._conn - 1]  # nel x nn x ncomp
        return np.ascontiguousarray(d.reshape(d.shape[0], -1))


def ndofsperel(it):
    return it.fesp.ndofsperel()


def eldofs(it):
    return it._dofs


def elnodes(it):
    return it._nodes


def eldofentmdims(it):
    return it._entmdim


def eldofcomps(it):
    return it._dofcomp


def eldofvals(it):
    """DOF values of the current element (src/FEIterators.jl:201-208)."""
    return it.fesp.field.dofvals[it._nodes - 1].ravel()


def jacjac(it, qpit):
    """(J, det J) at the current quadrature point (src/FEIterators.jl:218-220)."""
    X = it._geom[it._nodes - 1]  # nn x 2
    J = X.T @ qpit._geomgrad[qpit._pt]
    return J, J[0, 0] * J[1, 1] - J[1, 0] * J[0, 1]


def location(it, qpit):
    """Location of the current quadrature point (src/FEIterators.jl:227-235)."""
    X = it._geom[it._nodes - 1]
    return qpit._geomN[qpit._pt] @ X


class QPIterator:
    """Quadrature-point iterator over precomputed basis tables (src/QPIterators.jl:59-84)."""

    def __init__(self, fesp: FESpace, quadraturesettings=None):
        self.fesp = fesp
        self.quadr = quadrature(fesp.fe.refshape, quadraturesettings)
        fe = fesp.fe
        pc = self.quadr.param_coords
        bfn = edofbfnum(fesp) - 1
        self._scalN = np.array([fe.bfun(pc[q]) for q in range(self.quadr.npts)])
        self._scalG = np.array([fe.bfungradpar(pc[q]) for q in range(self.quadr.npts)])
        self._N = self._scalN[:, bfn]  # expanded to the vector element (src/QPIterators.jl:34-39)
        self._G = self._scalG[:, bfn, :]
        self._geomN = self._scalN
        self._geomgrad = self._scalG
        self._bfnum = bfn
        self._pt = 0

    def __len__(self):
        return self.quadr.npts

    def __iter__(self):
        for q in range(self.quadr.npts):
            self._pt = q
            yield self


def bfun(qp):
    return qp._N[qp._pt]


def bfungradpar(qp):
    return qp._G[qp._pt]


def bfungrad(qp, Jac):
    """Spatial gradients gradNpar / J (src/QPIterators.jl:132-140); ndofsperel x 2."""
    g = np.linalg.solve(np.asarray(Jac).T, qp._scalG[qp._pt].T).T
    return g[qp._bfnum]


def weight(qp):
    return qp.quadr.weights[qp._pt]


__all__ = ["FEIterator", "QPIterator", "eldofs", "elnodes", "eldofentmdims", "eldofcomps", "eldofvals", "jacjac",
           "location", "bfun", "bfungradpar", "bfungrad", "weight", "ndofsperel", "edofmdim", "edofcompnt"]
