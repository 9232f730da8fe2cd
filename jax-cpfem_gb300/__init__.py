"""GB300-native crystal-plasticity FE hot path: the per-Gauss-point Kalidindi update and
the HEX8 global Newton step (residual, consistent tangent, CSR assembly, BiCGSTAB) as
sm_103a CUDA behind the reference's ``CrystalPlasticity`` / ``solver`` interface.

The CUDA library (``libcpfem_gb300.so``, C ABI in ``include/cpfem_gb300.h``) is required;
importing the problem classes loads it and fails loudly if it has not been built.
"""
from . import material, mesh
from .material import MaterialSpec
from .mesh import Mesh, box_mesh

__all__ = ["material", "mesh", "MaterialSpec", "Mesh", "box_mesh", "load"]


def load():
    """Import the GPU modules (loads the CUDA library)."""
    from . import _capi, problem, solver  # noqa: F401
    _capi.load()
    return problem, solver
