"""GB300-native PolyDG elastodynamics hot path of LYMPH3D.

The compute path is liblymph3d_gb300.so (hand-written CUDA for sm_103a behind
the C ABI in include/lymph3d_gpu.h); this package is its host-side mirror of
the reference's matrix_free module.  Every entry point loads the library
(building it in-tree when nvcc is present) and raises if it is missing; there
is no CPU stand-in.
"""
from . import _lib
from ._lib import LymphError, load
from .matrix_free import MatrixFree, run_reference_driver, time_function
from .mesh import Mesh, cube, lognormal_materials, read_deck

__all__ = ["LymphError", "load", "MatrixFree", "run_reference_driver", "time_function", "Mesh", "cube",
           "lognormal_materials", "read_deck", "_lib"]
