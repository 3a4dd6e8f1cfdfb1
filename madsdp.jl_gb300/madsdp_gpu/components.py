"""Component selectors and options, mirroring MadSDP's component API.

Each class stands for the reference type of the same name in
src/components.jl (defaults included) and is marshalled into the
``msdp_components`` struct of the C ABI; ``Options`` mirrors
``MadSDPOptions`` (src/options.jl:3-15).
"""

from __future__ import annotations

import enum
import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

__all__ = [
    "Status", "NT", "HKM", "EigenStep", "CholeskyBacktrack", "Mehrotra", "AdaptiveMu",
    "PrimalDual", "DualCentering", "ScaledIdentity", "InitialPoint", "DualShift",
    "DenseCholesky", "MadNLPSchur", "QRSchur", "Options", "PRECISIONS",
]


class Status(enum.IntEnum):
    """MadNLP.Status values used by MadSDP (src/moi.jl:16-29)."""

    SOLVE_SUCCEEDED = 1
    SOLVED_TO_ACCEPTABLE_LEVEL = 2
    SEARCH_DIRECTION_BECOMES_TOO_SMALL = 3
    MAXIMUM_ITERATIONS_EXCEEDED = 5
    MAXIMUM_WALLTIME_EXCEEDED = 6
    INFEASIBLE_PROBLEM_DETECTED = 8
    ERROR_IN_STEP_COMPUTATION = 11
    USER_REQUESTED_STOP = 13
    INITIAL = 100
    REGULAR = 101

    def solvercore(self) -> str:
        """SolverCore status symbol (src/moi.jl:16-29)."""
        return {
            1: "first_order", 2: "acceptable", 3: "small_step", 5: "max_iter", 6: "max_time",
            8: "infeasible", 11: "exception", 13: "user",
        }.get(int(self), "unknown")


# --- search directions (src/components.jl:110-153) --------------------------

@dataclass(frozen=True)
class NT:
    """Nesterov-Todd direction: E(M) = W M W with W S W = X."""
    code = 0


@dataclass(frozen=True)
class HKM:
    """HKM direction: E(M) = (X M S^-1 + S^-1 M X) / 2."""
    code = 1


# --- step lengths (src/components.jl:156-193) --------------------------------

@dataclass(frozen=True)
class EigenStep:
    tau: float = 0.95
    code = 0


@dataclass(frozen=True)
class CholeskyBacktrack:
    shrink: float = 0.8
    boundary: float = 0.95
    code = 1


# --- centering (src/components.jl:196-235) -----------------------------------

@dataclass(frozen=True)
class Mehrotra:
    sigma_exponent: float = 3.0
    code = 0


@dataclass(frozen=True)
class AdaptiveMu:
    initial_ratio: float = 0.25
    ratio: float = 0.5
    code = 1


# --- algorithms (src/components.jl:51-108) -----------------------------------

@dataclass(frozen=True)
class PrimalDual:
    direction: object = field(default_factory=NT)
    step: object = field(default_factory=EigenStep)
    centering: object = field(default_factory=Mehrotra)
    code = 0


@dataclass(frozen=True)
class DualCentering:
    beta: float = 0.2
    delta: float = 1.0
    A: Optional[float] = 2.0
    centering_max_iter: int = 50
    code = 1


# --- initial points (src/components.jl:237-294) ------------------------------

class ScaledIdentity:
    """X = S = beta I, x = z = beta, y = 0; beta from the data if not given."""

    code = 0

    def __init__(self, scale: Optional[float] = None):
        if scale is not None:
            scale = float(scale)
            if not math.isfinite(scale) or scale <= 0:
                raise ValueError("The identity scale must be finite and positive.")
        self.scale = scale


@dataclass
class InitialPoint:
    X: Sequence[np.ndarray]
    y: np.ndarray
    x: Optional[np.ndarray] = None
    code = 1


@dataclass(frozen=True)
class DualShift:
    initial_shift: float = 1.0
    max_shift: float = 1e10
    code = 2


# --- Schur solvers (src/components.jl:296-343) -------------------------------

@dataclass(frozen=True)
class DenseCholesky:
    code = 0


@dataclass(frozen=True)
class MadNLPSchur:
    code = 1


@dataclass(frozen=True)
class QRSchur:
    code = 2


@dataclass
class Options:
    """MadSDPOptions (src/options.jl:3-15) plus the mixed-precision switch."""

    tol: float = 1e-7
    max_iter: int = 100
    max_wall_time: float = 3600.0
    mu_min: float = 1e-14
    regularize_schur: float = 1e-12
    max_schur_reg: int = 8
    datasparsity: int = 8
    # MSDP_MIXED: FP32 iterations while max(inf_pr, inf_du, gap) > switch_tol
    switch_tol: float = 0.0
    # MSDP_MIXED: refinement passes of each FP32 direction against the
    # float64 primal defect
    mixed_refine: int = 2


# "fp64_tensor": whole-GPU solver, FP64 products emulated on tensor cores
PRECISIONS = {"fp64": 0, "mixed": 1, "fp64_tensor": 2}
