"""FE fields and spaces: DOF storage and numbering.

Mirror of Elfel.jl src/FEFields.jl and src/FESpaces.jl with numpy arrays in
place of Vector{SVector}.  The numbering is the reference's, bit for bit:
free DOFs are numbered term-major / component-minor skipping data DOFs, data
DOFs afterwards in the same order (src/FEFields.jl:137-177), and several
spaces number all their free DOFs first, then all data DOFs
(src/FESpaces.jl:250-259).  Numbers are 1-based; 0 marks "not numbered".
Julia's ``name!`` functions are called ``name`` here.
"""
import numpy as np

from .felements import FE


class FEField:
    """Per-entity DOF numbers, datum flags and values (src/FEFields.jl:14-33)."""

    def __init__(self, ncomp, nterms, dtype=np.float64):
        self.dofnums = np.zeros((nterms, ncomp), dtype=np.int64)
        self.isdatum = np.zeros((nterms, ncomp), dtype=bool)
        self.dofvals = np.zeros((nterms, ncomp), dtype=dtype)

    def nterms(self):
        return self.dofnums.shape[0]

    def ndofsperterm(self):
        return self.dofnums.shape[1]

    def ndofs(self):
        return self.dofnums.size

    def doftype(self):
        return self.dofvals.dtype.type

    def setebc(self, tid, comp, val):
        """setebc!(f, tid, comp, val); tid and comp 1-based (scalars or arrays)."""
        t = np.asarray(tid, dtype=np.int64) - 1
        c = np.asarray(comp, dtype=np.int64) - 1
        self.isdatum[t, c] = True
        self.dofvals[t, c] = val
        return self

    def setdofval(self, tid, comp, val):
        t = np.asarray(tid, dtype=np.int64) - 1
        c = np.asarray(comp, dtype=np.int64) - 1
        self.dofvals[t, c] = val
        return self

    def numberfreedofs(self, firstnum=1):
        """numberfreedofs!(f, firstnum): src/FEFields.jl:137-154."""
        free = ~self.isdatum.ravel()
        n = np.zeros(self.dofnums.size, dtype=np.int64)
        n[free] = firstnum + np.arange(int(free.sum()), dtype=np.int64)
        self.dofnums = n.reshape(self.dofnums.shape)
        return self

    def numberdatadofs(self, firstnum=1):
        """numberdatadofs!(f, firstnum): src/FEFields.jl:164-177."""
        d = self.isdatum.ravel()
        n = self.dofnums.ravel().copy()
        n[d] = firstnum + np.arange(int(d.sum()), dtype=np.int64)
        self.dofnums = n.reshape(self.dofnums.shape)
        return self

    def _nums(self, mask):
        v = self.dofnums[mask]
        t = int(v.size)
        if t == 0:
            return (np.iinfo(np.int64).max, 0, 0)
        return (int(v.min()), int(v.max()), t)

    def freedofnums(self):
        """(first, last, total) of the free DOFs (src/FEFields.jl:187-201)."""
        return self._nums(~self.isdatum)

    def datadofnums(self):
        """(first, last, total) of the data DOFs (src/FEFields.jl:219-233)."""
        return self._nums(self.isdatum)

    def highestfreedofnum(self):
        return self.freedofnums()[1]

    def highestdatadofnum(self):
        return self.datadofnums()[1]

    def gathersysvec(self, vec):
        """vec[dofnums] = dofvals (src/FEFields.jl:247-257); vec indexed 1-based via the numbers."""
        n = self.dofnums.ravel()
        ok = n > 0
        vec[n[ok] - 1] = self.dofvals.ravel()[ok]
        return vec

    def scattersysvec(self, v):
        """dofvals = v[dofnums] where the number is within v (src/FEFields.jl:264-279)."""
        n = self.dofnums.ravel()
        ok = (n >= 1) & (n <= len(v))
        vals = self.dofvals.ravel().copy()
        vals[ok] = np.asarray(v)[n[ok] - 1]
        self.dofvals = vals.reshape(self.dofvals.shape)
        return self


class FESpace:
    """Mesh + scalar FE x nfecopies components (src/FESpaces.jl:25-40).

    One FEField per manifold dimension m that carries DOFs
    (ndofperfeat(fe, m) > 0; src/FESpaces.jl:73-83): m = 0 holds one term per
    mesh node, m = manifdim(fe) one term per element (the identity incidence
    relation of the cells, ``ir_identity`` in the reference's scripts).  The
    library's elements carry no DOFs on edges or faces.

    Fields are numbered in ascending m.  The reference iterates its
    Dict{Int} of fields (src/FESpaces.jl:141-173), whose order for the keys
    {0, 2} or {0, 3} is Julia's hash order; for spaces with a single field
    (all nodal and all cell-constant elements) the two agree.
    """

    def __init__(self, T, mesh, fe: FE, nfecopies=1):
        self.mesh = mesh
        self.fe = fe
        self.nfecopies = int(nfecopies)
        self.T = T
        if mesh.nodes_per_elem != fe.nodes_per_elem or (fe.shape != mesh.etype and mesh.etype in ("T3", "T6", "Q4",
                                                                                                   "T4", "L2")):
            raise ValueError(f"mesh of {mesh.etype} cells ({mesh.nodes_per_elem} nodes) for {fe}")
        self._fields = {}
        md = fe.manifdim()
        for m in range(0, md + 1):
            if fe.ndofperfeat(m) == 0:
                continue
            if m == 0:
                nterms = mesh.nnodes
            elif m == md:
                nterms = mesh.nel
            else:
                raise NotImplementedError(f"DOFs on features of dimension {m} of {fe}")
            self._fields[m] = FEField(self.nfecopies, nterms, dtype=T)  # one DOF per feature
        self._edofmdim, self._edofbfnum, self._edofcompnt = _number_edofs(fe, self.nfecopies)

    @property
    def field(self):
        """The nodal field (manifold dimension 0), or the only field of the space."""
        return self._fields[0] if 0 in self._fields else next(iter(self._fields.values()))

    def ndofsperel(self):
        return self.fe.ndofsperel() * self.nfecopies


def _number_edofs(fe, nfecopies):
    """Per element-DOF manifold dim, basis function number, component (src/FESpaces.jl:87-105)."""
    emdim, bfnum, compnt = [], [], []
    bfn = 1
    for m in range(0, 4):
        for _ in range(fe.nfeatofdim(m)):
            for _k in range(fe.ndofperfeat(m)):
                for j in range(1, nfecopies + 1):
                    emdim.append(m)
                    bfnum.append(bfn)
                    compnt.append(j)
                bfn += 1
    return np.array(emdim), np.array(bfnum), np.array(compnt)


def doftype(fesp):
    return fesp.T


def edofmdim(fesp):
    return fesp._edofmdim


def edofbfnum(fesp):
    return fesp._edofbfnum


def edofcompnt(fesp):
    return fesp._edofcompnt


def ndofsperel(fesp):
    return fesp.ndofsperel()


def dofnum(fesp, m, eid, comp):
    """DOF number of entity eid (1-based) of dimension m, component comp (src/FESpaces.jl:123-130)."""
    if fesp.fe.ndofperfeat(m) > 0 and m in fesp._fields:
        return int(fesp._fields[m].dofnums[eid - 1, comp - 1])
    return 0


def numberfreedofs(fesp, firstnum=1):
    for m, f in fesp._fields.items():
        f.numberfreedofs(firstnum)
        firstnum = f.freedofnums()[1] + 1
    return fesp


def numberdatadofs(fesp, firstnum=0):
    firstnum = nunknowns(fesp) + 1 if firstnum == 0 else firstnum
    for m, f in fesp._fields.items():
        f.numberdatadofs(firstnum)
        firstnum = f.datadofnums()[1] + 1
    return fesp


def ndofs(fesp):
    return sum(f.ndofs() for f in fesp._fields.values())


def nunknowns(fesp):
    return sum(f.freedofnums()[2] for f in fesp._fields.values())


def highestfreedofnum(fesp):
    return max([0] + [f.highestfreedofnum() for f in fesp._fields.values()])


def highestdatadofnum(fesp):
    return max([0] + [f.highestdatadofnum() for f in fesp._fields.values()])


def numberdofs(fesp):
    """numberdofs!(fesp) / numberdofs!([fesp1, fesp2, ...]) of src/FESpaces.jl:250-273."""
    spaces = list(fesp) if isinstance(fesp, (list, tuple)) else [fesp]
    numberfreedofs(spaces[0], 1)
    for i in range(1, len(spaces)):
        numberfreedofs(spaces[i], highestfreedofnum(spaces[i - 1]) + 1)
    numberdatadofs(spaces[0], highestfreedofnum(spaces[-1]) + 1)
    for i in range(1, len(spaces)):
        numberdatadofs(spaces[i], highestdatadofnum(spaces[i - 1]) + 1)
    return fesp


def setebc(fesp, m, eid, comp, val):
    """setebc!(fesp, m, eid, comp, val): eid/comp 1-based, scalars or arrays (src/FESpaces.jl:287-291)."""
    fesp._fields[m].setebc(eid, comp, val)
    return fesp


def setdofval(fesp, m, eid, comp, val):
    fesp._fields[m].setdofval(eid, comp, val)
    return fesp


def gathersysvec(v, fesp):
    """Fill v with the DOF values of one space or of a list of spaces (src/FESpaces.jl:316-337)."""
    for s in (fesp if isinstance(fesp, (list, tuple)) else [fesp]):
        for f in s._fields.values():
            f.gathersysvec(v)
    return v


def scattersysvec(fesp, v):
    """Copy a system vector back into the DOF values (src/FESpaces.jl:344-365)."""
    for s in (fesp if isinstance(fesp, (list, tuple)) else [fesp]):
        for f in s._fields.values():
            f.scattersysvec(v)
    return fesp


def makeattribute(fesp, name, comp):
    """Attribute of component(s) comp (1-based) over the entities of the space's
    first field (nodes, or cells for cell-constant elements): nterms x len(comp) values."""
    c = np.atleast_1d(np.asarray(comp)) - 1
    vals = fesp.field.dofvals[:, c]
    if not hasattr(fesp.mesh, "attributes"):
        fesp.mesh.attributes = {}
    fesp.mesh.attributes[name] = vals
    return vals
