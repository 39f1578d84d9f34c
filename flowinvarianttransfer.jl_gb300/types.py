"""Trait and result types mirroring FlowInvariantTransfer.jl's ``src/Types.jl``.

The names, fields and defaults follow the reference so that calls read the same:
binnings (``:370-411``), shell geometry (``:506-531``), dealiasing (``:458-476``), invariants
(``:77-132``), decompositions, spectral / execution backends (``:550-635``) and result structs
(``:654,719,746``). ``GB300Spectral`` and ``GB300Execution`` are the new backends that route a
call to the GB300 library.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Optional, Sequence, Tuple

import numpy as np


# ---- binning ------------------------------------------------------------------------------------
class AbstractShellBinning:
    pass


@dataclass(frozen=True)
class LinearBinning(AbstractShellBinning):
    dk: float


@dataclass(frozen=True)
class LogarithmicBinning(AbstractShellBinning):
    k0: float
    lam: float


@dataclass(frozen=True)
class DyadicBinning(AbstractShellBinning):
    k0: float = 1.0


@dataclass(frozen=True)
class CustomBinning(AbstractShellBinning):
    edges: Tuple[float, ...]

    def __init__(self, edges):
        object.__setattr__(self, "edges", tuple(float(e) for e in edges))


@dataclass(frozen=True)
class SmoothBands:
    """Graded log-Gaussian bands (``src/Types.jl:414-430``): centers > 0 increasing, logwidth in ln k."""
    centers: Tuple[float, ...]
    logwidth: float = 0.6

    def __init__(self, centers, logwidth=0.6):
        object.__setattr__(self, "centers", tuple(float(c) for c in centers))
        object.__setattr__(self, "logwidth", float(logwidth))


# ---- shell geometry -----------------------------------------------------------------------------
@dataclass(frozen=True)
class ShellMagnitude:
    """Bin by sqrt(sum_{d in dims} k_d^2); ``dims=None`` = all axes. dims are 1-based."""
    dims: Optional[Tuple[int, ...]] = None


def IsotropicShells():
    return ShellMagnitude(None)


def PerpendicularShells(dims=(1, 2)):
    return ShellMagnitude(tuple(dims))


def ParallelShells(dims=(3,)):
    return ShellMagnitude(tuple(dims))


# ---- dealiasing ---------------------------------------------------------------------------------
class AbstractDealiasing:
    key = ""


class NoDealiasing(AbstractDealiasing):
    key = "none"


class OrszagTwoThirds(AbstractDealiasing):
    key = "two_thirds"


class PaddedThreeHalves(AbstractDealiasing):
    key = "three_halves"


# ---- invariants ---------------------------------------------------------------------------------
class AbstractInvariant:
    code = -1


class KineticEnergy(AbstractInvariant):
    code = 0


class PassiveScalar(AbstractInvariant):
    code = 1


class Helicity(AbstractInvariant):
    code = 2


class Enstrophy(AbstractInvariant):
    code = 3


# ---- decompositions -----------------------------------------------------------------------------
class AbstractFieldDecomposition:
    pass


class NoDecomposition(AbstractFieldDecomposition):
    pass


class HelicalDecomposition(AbstractFieldDecomposition):
    names = ("positive", "negative")


class HelmholtzDecomposition(AbstractFieldDecomposition):
    names = ("rotational", "divergent")


class ToroidalPoloidalDecomposition(AbstractFieldDecomposition):
    """Craya-Herring toroidal / poloidal split (``src/Decomposition.jl:107-141``, 3D)."""
    names = ("toroidal", "poloidal")


class RotationalDecomposition(AbstractFieldDecomposition):
    pass


class DivergentDecomposition(AbstractFieldDecomposition):
    pass


# ---- filters (src/Types.jl filter types, src/Filters.jl:19-26) ----------------------------------
class AbstractFilter:
    code = -1


class SharpSpectralFilter(AbstractFilter):
    code = 0


class GaussianFilter(AbstractFilter):
    code = 1


class TopHatFilter(AbstractFilter):
    code = 2


# ---- backends -----------------------------------------------------------------------------------
class AbstractSpectralBackend:
    pass


@dataclass(frozen=True)
class GB300Spectral(AbstractSpectralBackend):
    """Transforms and products on the GB300. ``precision`` 64 (the plain FP64 method) or 32
    (FP32 transforms/products, FP64 reductions); ``None`` follows the input element type."""
    precision: Optional[int] = None


class FFTBackend(AbstractSpectralBackend):
    """Accepted for drop-in calls: routed to ``GB300Spectral()``."""


class DirectSumBackend(AbstractSpectralBackend):
    """Accepted for drop-in calls: routed to ``GB300Spectral()`` (same arithmetic, O(N log N))."""


class AbstractExecutionBackend:
    pass


@dataclass(frozen=True)
class GB300Execution(AbstractExecutionBackend):
    """How the shell-to-shell mediator loop runs: ``"batched"`` (mediators batched, fused
    kernels, CUDA-graph replay) or ``"plain"`` (one nonlinear term per mediator, launched one
    by one, as the reference's serial loop)."""
    mode: str = "batched"


class SerialBackend(AbstractExecutionBackend):
    pass


class ThreadedBackend(AbstractExecutionBackend):
    pass


# ---- methods (unified dispatch, src/Types.jl) ---------------------------------------------------
@dataclass(frozen=True)
class SpectralFluxMethod:
    binning: AbstractShellBinning


@dataclass(frozen=True)
class ShellToShellTransferMethod:
    binning: AbstractShellBinning


@dataclass(frozen=True)
class ModeToModeTransferMethod:
    """``ModeToModeTransferMethod(; binning=nothing, invariant=KineticEnergy())`` (``src/Types.jl:288-295``)."""
    binning: Any = None
    invariant: Any = None


@dataclass(frozen=True)
class CoarseGrainingFluxMethod:
    """``CoarseGrainingFluxMethod(filter, scale)`` (``src/Types.jl:241-244``): the filter kernel and
    its length scale ell."""
    filter: Any
    scale: float


# ---- results ------------------------------------------------------------------------------------
@dataclass
class SpectralFluxResult:
    k_shells: np.ndarray
    transfer_spectrum: np.ndarray
    flux: np.ndarray


@dataclass
class ShellToShellResult:
    shell_centers: np.ndarray
    shell_edges: np.ndarray
    transfer_matrix: np.ndarray
    net_transfer: np.ndarray
    max_antisymmetry_error: float


@dataclass
class ModeToModeTriadResult:
    invariant: AbstractInvariant
    ks: Any
    net_transfer: np.ndarray
    transfer: np.ndarray


@dataclass
class PartialFluxResult:
    channels: dict
    total: SpectralFluxResult
    k_shells: np.ndarray


@dataclass
class CoarseGrainingFluxResult:
    """src/Types.jl:673-677."""
    filter_scale: float
    flux_field: np.ndarray
    mean_flux: float


@dataclass
class CoarseGrainingFluxResultWithDiagnostics:
    """src/Types.jl:681-: the flux plus the subfilter stress tau_ij and filtered strain S_ij,
    each of shape (ns..., nd, nd)."""
    filter_scale: float
    flux_field: np.ndarray
    mean_flux: float
    tau: np.ndarray
    strain: np.ndarray


@dataclass
class BandToBandResult:
    """The NamedTuple of ``calculate_band_to_band_transfer`` (``src/BandTransfer.jl:109-111``)."""
    centers: np.ndarray
    transfer_matrix: np.ndarray
    net_transfer: np.ndarray
    max_antisymmetry_error: float
