"""clawpack_gb300 -- PyClaw's classic unsplit 2D wave-propagation step on
NVIDIA GB300 (sm_103a).

Subpackages:
  pyclaw   PyClaw-compatible API (Controller, ClawSolver2D, State, ...)
  riemann  descriptors of the supported Riemann solvers
  device   device-resident state and the C-ABI wrappers of libgclaw.so
  workloads  the initial/boundary data of the benchmark problems

The compute path is libgclaw.so (CUDA); importing the package does not load
it, calling a solver does, and fails loudly if it has not been built.
"""
__version__ = "0.1.0"
