"""GB300 interior-point library for MadSDP: host-side mirror of its API.

The numerical work runs in libmadsdp_gpu.so (sm_103a); this package only
marshals models, component selectors and options across the C ABI.
"""

from .components import (AdaptiveMu, CholeskyBacktrack, DenseCholesky, DualCentering, DualShift,
                         EigenStep, HKM, InitialPoint, MadNLPSchur, Mehrotra, NT, Options,
                         PrimalDual, QRSchur, ScaledIdentity, Status)
from .model import BlockConstraints, Model
from .solver import (Batch, Context, GPUError, InstanceSolver, MadSDPSolver, SchurWorkspace, default_context,
                     madsdp)

__all__ = [
    "AdaptiveMu", "Batch", "BlockConstraints", "CholeskyBacktrack", "Context", "DenseCholesky",
    "DualCentering", "DualShift", "EigenStep", "GPUError", "HKM", "InitialPoint", "InstanceSolver", "MadNLPSchur",
    "SchurWorkspace", "MadSDPSolver", "Mehrotra", "Model", "NT", "Options", "PrimalDual", "QRSchur",
    "ScaledIdentity", "Status", "default_context", "madsdp",
]
