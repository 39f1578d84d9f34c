"""GB300-native transfer hot path of FlowInvariantTransfer.jl (imported as ``fit_gb300``).

Python host mirror of the reference API over libfit_gb300.so (hand-written CUDA for sm_103a):
the pseudospectral nonlinear term with 2/3 or 3/2 dealiasing and the shell-binned reductions
built on it — spectral flux, shell-to-shell, partial fluxes, mode-to-mode — plus the
coarse-graining flux, a forced Navier-Stokes evolver and the learned subfilter-stress closure.
"""
from .types import *  # noqa: F401,F403
from .shells import (wavenumber_grid, wavenumber_magnitude_grid, dealiasing_mask, shell_edges,  # noqa: F401
                     shell_centers, n_shells, default_binning, kmax, dims_mask)
from .api import (compute_nonlinear_term, transfer_density, decompose_field, assign_shells_device,  # noqa: F401
                  calculate_spectral_flux, calculate_scalar_flux, calculate_shell_to_shell_transfer,
                  calculate_scalar_shell_to_shell_transfer, calculate_partial_fluxes,
                  calculate_helical_partial_fluxes, calculate_partial_fluxes_multi, calculate_mode_to_mode_transfer,
                  calculate_scalar_mode_to_mode_transfer, calculate_energy_transfer,
                  calculate_band_to_band_transfer, physical_to_spectral)
from .plan import Plan, get_plan, clear_plans  # noqa: F401
from .batch import (SpectralFluxBatch, calculate_spectral_flux_batch, autotune_summary,  # noqa: F401
                    autotune_enable, autotune_clear)
from .closure import (calculate_coarse_graining_flux, evolve_forced_navier_stokes,  # noqa: F401
                      evolve_forced_navier_stokes_device, closure_data, ClosureData, SubfilterStressMLP,
                      gradient_model_flux, field_compare)
from .replicas import mpi_batch_map, batch_map  # noqa: F401
from . import _lib  # noqa: F401
from ._lib import FitError, launch_count, lib_path  # noqa: F401
