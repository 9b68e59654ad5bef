"""GB300-native finite-element assembly + solve for the GradientRobustMultiPhysics.jl hot path.

The compute path is libgrmp_gpu.so (C-ABI in include/grmp.h, CUDA kernels for
sm_103a in csrc/); this package is the host-side mirror of the reference's
interface (meshes, FE spaces, operators, FEMatrix / FEVector, assemble!,
solve!) over that C-ABI.
"""
from .mesh import SimplexMesh, grid_unitsquare, grid_unitcube_kuhn  # noqa: F401
from .fespace import (FESpace, FEType, H1P1, H1P2, H1BR, H1P2B, L2P0, HDIVRT0, HDIVBDM1, HDIVRT1,  # noqa: F401
                      HDIVBDM2, FE_H1P1, FE_H1P2, FE_H1BR, FE_H1P2B, FE_L2P0, FE_HDIVRT0, FE_HDIVBDM1)
from . import _lib  # noqa: F401
from .api import (GB300Context, Operator, CellCoefficient, LaplaceOperator, ReactionOperator,  # noqa: F401
                  HookStiffnessOperator2D, HookStiffnessOperator3D, BilinearForm, LinearForm, DataFunction,
                  FEMatrix, FEVector, ImportedMatrix, assemble, apply_dirichlet, GB300PCG, spmv,
                  Identity, Gradient, SymmetricGradient, Divergence, ReconstructionIdentity,
                  ReconstructionIdentityBDM1, ReconstructionIdentityRT1, ReconstructionIdentityBDM2,
                  ReconstructionDivergence, APT_BilinearForm, APT_SymmetricBilinearForm,
                  ItemIntegrator, L2ErrorIntegrator, L2NormIntegrator, L2DifferenceIntegrator,
                  NonlinearForm, StructuralCoupling, assemble_nonlinear, solve_nonlinear,
                  Jump, ON_CELLS, ON_IFACES, FaceVolumePower, FaceJumpIntegrator)
from .fespace import interpolate  # noqa: F401
from ._lib import FP64, FP32, FP64_FP32, DIRICHLET_PENALTY, DIRICHLET_ELIMINATE, GrmpError  # noqa: F401

__version__ = "0.1.0"
