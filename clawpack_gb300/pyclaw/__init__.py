"""PyClaw-compatible front end of the GB300 classic 2D step.

``from clawpack_gb300 import pyclaw, riemann`` gives the names user scripts
take from ``clawpack.pyclaw`` and ``clawpack.riemann`` for the classic
unsplit 2D path: Controller, Solution, State, Domain, Dimension,
ClawSolver2D, BC and limiters.tvd.
"""
from . import limiters  # noqa: F401
from .controller import Controller  # noqa: F401
from .geometry import Dimension, Domain, Grid, Patch  # noqa: F401
from .solver import BC, ClawSolver2D, ClawSolver3D  # noqa: F401
from .state import Solution, State  # noqa: F401
