"""cylag_gb300: CyLag's per-particle time step as one fused sm_103a kernel.

Drop-in for the cylag.core API on the particle-step path:
``TriangularMesh``, ``EulerianFieldSet``, ``LagrangianParticleSet``,
``Solver`` keep the reference's signatures; the particle loop runs on the
GPU through libcylag_gpu.so (C ABI in include/cylag_gpu.h).
"""
from .core import EulerianFieldSet, LagrangianParticleSet, SimuTime, Solver
from .mesh import TriangularMesh
from .parameters import CYLAG_DEFAULT_PARAMETERS, Parameters

__all__ = ["TriangularMesh", "EulerianFieldSet", "LagrangianParticleSet", "Solver",
           "SimuTime", "Parameters", "CYLAG_DEFAULT_PARAMETERS"]
__version__ = "0.1.0"
