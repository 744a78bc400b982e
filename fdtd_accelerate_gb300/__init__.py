"""GB300-native 3D FDTD (Maxwell) Yee time step.

Hot path: the 2nd-order Yee step (update_e / update_h curl stencils, CPML
psi updates on the absorbing slabs, soft sources) and the 4th-order
symplectic variant, as hand-written sm_103a CUDA kernels behind the C ABI
in include/fdtd_gb300.h, with the reference's Python call shapes on top.
"""
from . import _native
from .batch import BatchSolver
from .adjoint import YeeAdjoint, fdtd_run
from .api import update_e, update_h, update_pbc_e, update_pbc_h
from .cpml import CpmlLayer, cpml_tables
from .drude import DrudeAde, drude_coefficients
from .tfsf import Tfsf
from .output import Output
from .solver import YeeSolver
from .sources import PointSources, gaussian_sine

__all__ = ["update_e", "update_h", "update_pbc_e", "update_pbc_h", "CpmlLayer", "cpml_tables", "DrudeAde",
           "drude_coefficients", "Tfsf", "Output",
           "YeeSolver", "BatchSolver", "YeeAdjoint", "fdtd_run", "PointSources", "gaussian_sine", "build"]


def build(force=False, verbose=False):
    from .buildlib import build as _b
    return _b(force=force, verbose=verbose)
