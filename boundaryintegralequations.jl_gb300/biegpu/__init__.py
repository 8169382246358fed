"""biegpu - GB300-native collocation BEM hot path of BoundaryIntegralEquations.jl.

The compute path is libbiegpu.so (CUDA, sm_103a) behind a C ABI
(include/biegpu.h); this package is its Python host side, mirroring the
reference's Julia API for the path:

  * ``Mesh3d`` and mesh builders (:mod:`biegpu.mesh`)
  * ``assemble_parallel`` -> (F, G, C)  (:mod:`biegpu.assembly`)
"""
from ._capi import BIEError, lib, library_path  # noqa: F401
from .assembly import (Context, assemble_parallel, basis, element_slicing, get_context,  # noqa: F401
                       quadrature_rule)
from .mesh import Mesh3d, ellipsoid, icosphere, load_comsol, read_comsol  # noqa: F401
from .operators import (Diagonal, FMMFOperator, FMMGOperator, GPUFOperator, GPUGOperator, I,  # noqa: F401
                        UniformScaling, gmres)
from .sweep import sweep  # noqa: F401
from .multisolve import solve_multi  # noqa: F401
from .adjoint import farfield_objective  # noqa: F401
from .rosebem import apply_taylor_expansion, taylor_assemble  # noqa: F401
from .lossy import (LossyGlobalOuter, ambient_to_properties, tangential_derivatives,  # noqa: F401
                    visco_thermal_constants)
from .distributed import sharded_sweep  # noqa: F401

__version__ = "0.1.0"
