"""Oracle for the structured-grid finite-volume step — TEST INFRASTRUCTURE ONLY.

This package is a CPU restatement, in NumPy, of TORCH's Cartesian
MUSCL-Hancock/HLLC step (python/cfdSolver/torchSolver2D.py,
python/cfdSolver/torchSolver3D.py, python/cfdSolver/torchFlux.py), its CFL
time step and session loop (python/cfdSolver/torchSession.py), the 1D chain
(python/cfdSolver/torchSolver.py) and the Arrhenius/ZND source.  Each function
cites the reference lines whose arithmetic it restates; the operation order is
kept identical so that an IEEE-754 double implementation without fused
multiply-add reproduces it bit for bit.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this package, and only as the checker or as the timed
CPU baseline.  The GPU library (``torch_gb300``) never imports it.

Pinning: ``tests/golden/make_golden.py`` runs the reference itself (imported
from its source tree in the development container) on small seeded inputs and
stores inputs and outputs under ``tests/golden/``; ``tests/test_oracle_golden.py``
checks this restatement against those vectors bit for bit.  The
nondimensional Arrhenius closure (T = p/rho, constant gamma) has no reference
implementation: parity for that closure is unpinned.
"""

from . import fv  # noqa: F401
from .session import OracleSimulation  # noqa: F401
