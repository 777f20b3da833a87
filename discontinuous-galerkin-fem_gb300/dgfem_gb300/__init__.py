"""GB300-native explicit DG residual-and-update path for compressible Euler and
Navier-Stokes (drop-in for dgfem's DGAssembler / SSP-RK3 path).  The compute lives in
libdgx.so (include/dgx.h); this package is its Python front end."""

from ._lib import DGXError, DGXInvalidArgument, DGXOutOfRange, LIB_PATH, load
from .api import (BCTypeEuler, BoundaryConditionEuler, CompressibleDGSolverBase, DGAssembler, DGBatch,
                  DGContext, DGMesh, DGSpace, EulerDGSolver, EulerWeakFormulation,
                  NavierStokesDGSolver, NavierStokesWeakFormulation, conserved_to_primitive,
                  kinetic_energy, primitive_to_conserved, rk3_trajectory)
from .vtk import VTKWriter

__all__ = ["DGXError", "DGXInvalidArgument", "DGXOutOfRange", "LIB_PATH", "load",
           "BCTypeEuler", "BoundaryConditionEuler", "CompressibleDGSolverBase", "DGAssembler", "DGBatch",
           "DGContext", "DGMesh", "DGSpace", "EulerDGSolver", "EulerWeakFormulation",
           "NavierStokesDGSolver", "NavierStokesWeakFormulation", "conserved_to_primitive",
           "primitive_to_conserved", "kinetic_energy", "rk3_trajectory", "VTKWriter"]
