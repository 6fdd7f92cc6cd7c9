"""oceananigans_gb300: GB300-native NonhydrostaticModel time stepping behind a C ABI.

The compute path is libgb300ocean.so (hand-written sm_103a CUDA); this package
is the host-side mirror of the reference's model API.
"""
from .api import (  # noqa: F401
    Periodic, Bounded, Flat,
    RectilinearGrid, ImmersedBoundaryGrid, GridFittedBottom,
    WENO, Smagorinsky, SmagorinskyLilly, AnisotropicMinimumDissipation, DynamicSmagorinsky, LagrangianAveraging, ScalarDiffusivity, BuoyancyTracer, FPlane,
    QuasiAdamsBashforth2TimeStepper,
    FluxBoundaryCondition, FieldBoundaryConditions,
    FFTBasedPoissonSolver, FourierTridiagonalPoissonSolver, ConjugateGradientPoissonSolver,
    NonhydrostaticModel, Ensemble, Simulation, set_, time_step_, run_,
    TimeStepWizard, conjure_time_step_wizard_, cell_advection_timescale, cell_diffusion_timescale,
)
from ._lib import GboError, NaNError, NotConvergedError, load  # noqa: F401
