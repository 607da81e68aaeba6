"""vonkarman_gb300 -- GB300-native (sm_103a) periodic pseudospectral step of
vonkarman, behind that project's own API for the path (FftBackend,
SpectralOps-based stepper, Tier-1 and Tier-2 diagnostics).

The compute path is libvonkarman_gpu.so (hand-written CUDA + C ABI); this
package only binds it.  Importing the solver classes does not need a GPU;
constructing one does, and fails loudly without the library or a device.
"""

from .solver import (  # noqa: F401
    GridSpec,
    GpuFftBackend,
    Periodic3D,
    ScalarDiagnostics,
    SolverOptions,
    SpectralOps,
    apply_viscous,
    compensated_spectrum,
    compute_nonlinear,
    create_backend,
    dissipation_spectrum,
    energy_spectrum,
    l2_inner,
    nonlinear_adjoint,
    spectral_ops,
)
from . import ics  # noqa: F401

__all__ = ["GridSpec", "GpuFftBackend", "Periodic3D", "ScalarDiagnostics", "SolverOptions", "SpectralOps",
           "apply_viscous", "spectral_ops",
           "compensated_spectrum", "compute_nonlinear", "create_backend", "dissipation_spectrum",
           "energy_spectrum", "ics", "l2_inner", "nonlinear_adjoint"]
