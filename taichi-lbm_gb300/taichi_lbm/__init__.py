"""GB300 (sm_103a) drop-in for taichi-lbm's per-step D2Q9 path.

Exports the reference package's public names (taichi_lbm/__init__.py of
taichi-lbm) with the same constructors and methods; every per-step method is
a CUDA kernel reached through the C ABI in include/lbm_gb300.h.  Additions:
FusedSolver (the whole step as one kernel per time step), Batch (many
lattices advanced together) and UnsupportedComposition.
"""
from . import _capi
from .lbm import LBField, MacroscopicEngine
from .boundary import (BoundarySpec, BoundaryClassifier, VelocityBB, VelocityEquilibrium,
                       VelocityNEEM, PressureABC, PressureNEEM, InsideBoundary, BoundaryEngine,
                       BounceBackWall, FluidBoundary, PeriodicAllBoundary, OpenNeumann,
                       OpenExtrapolation, OpenConvective1order, OpenConvective2order, MaskAndGroup)
from .collision import (BGKCollision, TRTCollision, MRTCollision, HuangMRTCollision,
                        PowerLawFluid, NewtonianFluid)
from .ibm import IBMNodes, Sphere, SphereIB, IBDEMCouplerEngine, IBEngine
from .shanchen import (ShanChenForceC1, ShanChenForceC2, BoundaryEngineSC, OpenNeumannPsi,
                       OpenConvective1orderPsi, OpenConvective2orderPsi, OpenExtrapolationPsi,
                       PeriodicPsi_LR, PeriodicPsi_BT, FixedPsi, SC_psi, vdW_psi, RK_psi, PR_psi,
                       CS_psi)
from .post import PostProcessingEngine
from .solver import FusedSolver
from .batch import Batch
from .serving import Request, Server
from .autotune import Autotuner
from ._plan import UnsupportedComposition

_capi.load()
