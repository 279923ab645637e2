"""GB300-native structured-grid finite-volume step for TORCH sessions.

Drop-in GPU path for the Cartesian MUSCL-Hancock / HLLC step of TORCH
(BFG508/TORCH, python/cfdSolver): hand-written CUDA kernels for sm_103a
behind a C ABI (include/tfv.h, libtfv.so) with a Python host layer that
mirrors the reference's session and step-function interfaces.
"""

from . import _lib  # noqa: F401
from .session import Simulation  # noqa: F401
from .stepfn import (hllc_flux, hllc_flux_grid, rusanov_flux, rusanov_flux_grid,  # noqa: F401
                     muscl_hancock_step_2d,
                     muscl_hancock_step_3d)

__all__ = ["Simulation", "hllc_flux", "hllc_flux_grid", "rusanov_flux", "rusanov_flux_grid",
           "muscl_hancock_step_2d",
           "muscl_hancock_step_3d"]
