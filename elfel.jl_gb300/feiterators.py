"""Element and quadrature-point iterators.

Mirror of Elfel.jl src/FEIterators.jl and src/QPIterators.jl.  Besides the
per-element iteration of the reference (used by user-written weak forms in
COO mode), FEIterator exposes the whole element DOF table at once
(``eldofs_table``), which is what the fused device assembly consumes.
"""
import numpy as np

from .felements import Jacobian
from .fespaces import FESpace, edofbfnum, edofcompnt, edofmdim
from .refshapes import quadrature


class FEIterator:
    """Iterates the elements of a space; caches nodes and DOF numbers (src/FEIterators.jl:34-82).

    The element's DOFs are those of its nodes (node-major, component-minor)
    followed by those of the cell itself (bubble and cell-constant
    elements), the order of _storedofs! over the fields of dimension
    0, 1, 2, 3 (src/FEIterators.jl:175-194).
    """

    def __init__(self, fesp: FESpace):
        self.fesp = fesp
        self._conn = fesp.mesh.conn
        self._geom = fesp.mesh.xy
        self._state = 0
        self._nodes = np.zeros(fesp.fe.nodes_per_elem, dtype=np.int64)
        self._dofs = np.zeros(fesp.ndofsperel(), dtype=np.int64)
        self._dofvals = np.zeros(fesp.ndofsperel(), dtype=fesp.T)
        # _init_e_d! (src/FEIterators.jl:155-166): entity dimension and component of each element DOF
        md, comps = [], []
        for m, f in fesp._fields.items():
            nent = fesp.fe.nodes_per_elem if m == 0 else 1
            md += [m] * (nent * f.ndofsperterm())
            comps += list(range(1, f.ndofsperterm() + 1)) * nent
        self._entmdim = np.array(md, dtype=np.int64)
        self._dofcomp = np.array(comps, dtype=np.int64)

    def __len__(self):
        return self._conn.shape[0]

    def __iter__(self):
        for e in range(len(self)):
            self._update(e + 1)
            yield self

    def _terms(self, m, state):
        return self._nodes - 1 if m == 0 else np.array([state - 1])

    def _update(self, state):
        """Cache the element's nodes and DOFs (src/FEIterators.jl:161-194)."""
        self._state = state
        self._nodes[:] = self._conn[state - 1]
        p = 0
        for m, f in self.fesp._fields.items():
            d = f.dofnums[self._terms(m, state)].ravel()
            self._dofs[p:p + d.size] = d
            p += d.size
        return self

    def eldofs_table(self):
        """All elements' DOF numbers (nel x ndofsperel, 1-based), in the order of eldofs."""
        parts = []
        for m, f in self.fesp._fields.items():
            if m == 0:
                d = f.dofnums[self._conn - 1]  # nel x nn x ncomp
                parts.append(d.reshape(d.shape[0], -1))
            else:
                parts.append(f.dofnums)  # nel x ncomp
        return np.ascontiguousarray(np.concatenate(parts, axis=1) if len(parts) > 1 else parts[0])


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
    """DOF values of the current element, in the order of eldofs (src/FEIterators.jl:201-208)."""
    p = 0
    for m, f in it.fesp._fields.items():
        v = f.dofvals[it._terms(m, it._state)].ravel()
        it._dofvals[p:p + v.size] = v
        p += v.size
    return it._dofvals


def jacjac(it, qpit):
    """(J, Jacobian) at the current quadrature point (src/FEIterators.jl:218-220):
    J = sum over the element's nodes of x_j (x) gradNpar_j of the geometry carrier."""
    nn = len(it._nodes)
    X = it._geom[it._nodes - 1]  # nn x sdim
    J = X.T @ qpit._geomgrad[qpit._pt][:nn]
    return J, Jacobian(J)


def location(it, qpit):
    """Location of the current quadrature point (src/FEIterators.jl:227-235)."""
    nn = len(it._nodes)
    X = it._geom[it._nodes - 1]
    return qpit._geomN[qpit._pt][:nn] @ X


class QPIterator:
    """Quadrature-point iterator over precomputed basis tables (src/QPIterators.jl:14-84).

    Basis values and parametric gradients of the scalar element are expanded
    to the element's DOFs through edofbfnum; the geometry is mapped with the
    element's geometry carrier (its own nodal basis, or the nodal element of
    the same shape for cell-constant elements).
    """

    def __init__(self, fesp: FESpace, quadraturesettings=None):
        self.fesp = fesp
        self.quadr = quadrature(fesp.fe.refshape, quadraturesettings)
        fe = fesp.fe
        gc = fe.geometrycarrier()
        pc = self.quadr.param_coords
        bfn = edofbfnum(fesp) - 1
        self._scalN = np.array([fe.bfun(pc[q]) for q in range(self.quadr.npts)])
        self._scalG = np.array([fe.bfungradpar(pc[q]) for q in range(self.quadr.npts)])
        self._N = self._scalN[:, bfn]  # expanded to the vector element (src/QPIterators.jl:34-39)
        self._G = self._scalG[:, bfn, :]
        self._geomN = np.array([gc.bfun(pc[q]) for q in range(self.quadr.npts)])
        self._geomgrad = np.array([gc.bfungradpar(pc[q]) for q in range(self.quadr.npts)])
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
    """Spatial gradients gradNpar / J (src/QPIterators.jl:132-140); ndofsperel x sdim.

    Right division by the square Jacobian matrix: g J = gradNpar."""
    J = np.atleast_2d(np.asarray(Jac, dtype=np.float64))
    g = np.linalg.solve(J.T, qp._scalG[qp._pt].T).T
    return g[qp._bfnum]


def weight(qp):
    return qp.quadr.weights[qp._pt]


__all__ = ["FEIterator", "QPIterator", "eldofs", "elnodes", "eldofentmdims", "eldofcomps", "eldofvals", "jacjac",
           "location", "bfun", "bfungradpar", "bfungrad", "weight", "ndofsperel", "edofmdim", "edofcompnt"]
