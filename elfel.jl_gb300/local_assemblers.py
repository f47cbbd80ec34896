"""Element-local matrix and vector assemblers (mirror of Elfel.jl src/LocalAssemblers.jl)."""
import numpy as np


class LocalMatrixAssembler:
    """Element matrix with the global row/col numbers of each entry (src/LocalAssemblers.jl:13-27).

    Stored column-major (Fortran order) like the Julia matrices, so the flat
    order of row/col/M is the order assemble! appends triplets in.
    """

    def __init__(self, nrow, ncol, z=0.0):
        self.row = np.zeros((nrow, ncol), dtype=np.int64, order="F")
        self.col = np.zeros((nrow, ncol), dtype=np.int64, order="F")
        self.M = np.full((nrow, ncol), z, dtype=np.float64, order="F")

    @property
    def shape(self):
        return self.M.shape

    def size(self):
        return self.M.shape

    def __getitem__(self, ij):
        i, j = ij
        return self.M[i - 1, j - 1]

    def __setitem__(self, ij, v):
        i, j = ij
        self.M[i - 1, j - 1] = v


class LocalVectorAssembler:
    """Element vector with its global row numbers (src/LocalAssemblers.jl:95-108)."""

    def __init__(self, nrow, z=0.0):
        self.row = np.zeros(nrow, dtype=np.int64)
        self.V = np.full(nrow, z, dtype=np.float64)

    def size(self):
        return self.V.shape

    def __getitem__(self, i):
        return self.V[i - 1]

    def __setitem__(self, i, v):
        self.V[i - 1] = v


class Transpose:
    """transpose(lma): assemble! appends the parent's entries with rows and columns swapped."""

    def __init__(self, parent):
        self.parent = parent


def transpose(lma):
    return Transpose(lma)


def init(a, rdofs, cdofs=None):
    """init!(lma, rdofs, cdofs) / init!(lva, rdofs): set numbers, zero values (src/LocalAssemblers.jl:68-83, 148-152)."""
    if isinstance(a, LocalMatrixAssembler):
        r = np.asarray(rdofs, dtype=np.int64).ravel()
        c = np.asarray(cdofs, dtype=np.int64).ravel()
        a.row[:, :] = r[:, None]
        a.col[:, :] = c[None, :]
        a.M[:, :] = 0.0
    else:
        a.row[:] = np.asarray(rdofs, dtype=np.int64).ravel()
        a.V[:] = 0.0
    return a
