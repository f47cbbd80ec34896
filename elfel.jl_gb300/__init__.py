"""GB300-native element integration, sparse assembly and sparse solve behind
Elfel.jl's assembly API.

The package is imported as ``elfel_gb300`` (its directory name holds a dot);
``__graft_entry__.package()`` at the repository root loads it.  The compute
path is libelfel_gpu.so (hand-written CUDA for sm_103a, C ABI in
include/elfel_gpu.h); this Python layer mirrors the reference's host API so
that scripts written against Elfel.jl translate line by line.
"""
from . import _native
from .assemblers import (SysmatAssemblerGPU, SysmatAssemblerSparse, SysvecAssembler, assemble, assemble_elasticity,
                         assemble_heat, assemble_stokes, finish, numberdofs_device, solve, start)
from .batching import BatchSolver
from .serving import HeatServer, heat_request
from .feiterators import (FEIterator, QPIterator, bfun, bfungrad, bfungradpar, eldofcomps, eldofentmdims, eldofs,
                          eldofvals, elnodes, jacjac, location, weight)
from .felements import (FEH1_L2, FEH1_Q4, FEH1_T3, FEH1_T3_BUBBLE, FEH1_T4, FEH1_T6, FEL2_Q4, FEL2_T3, FEL2_T4,
                        Jacobian, manifdim, nfeatofdim, ndofperfeat, ndofsperel as fe_ndofsperel, refshape, shapedesc)
from .fespaces import (FEField, FESpace, dofnum, doftype, edofbfnum, edofcompnt, edofmdim, gathersysvec,
                       highestdatadofnum, highestfreedofnum, makeattribute, ndofs, ndofsperel, numberdatadofs,
                       numberdofs, numberfreedofs, nunknowns, scattersysvec, setdofval, setebc)
from .local_assemblers import LocalMatrixAssembler, LocalVectorAssembler, init, transpose
from .meshes import (L2block, Mesh, Q4block, T3block, T4block, T6block, T6toT3, boundary_edges, boundary_nodes, jitter,
                     vselect, vselect_nearest)
from .refshapes import (IntegRule, RefShapeCube, RefShapeInterval, RefShapePoint, RefShapeSquare, RefShapeTetrahedron,
                        RefShapeTriangle, npts, param_coords, quadrature, weights)
from ._native import Context, ElfelError, NotConverged, default_context


def build(verbose=False):
    """Compile libelfel_gpu.so for sm_103a (nvcc) and load it."""
    import importlib

    _b = importlib.import_module(__name__ + ".nvcc_build")
    path = _b.build(verbose=verbose)
    _native.load()
    return path
