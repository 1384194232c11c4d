"""State and Solution with PyClaw's names (upstream pyclaw/src/pyclaw/state.py
and solution.py; absent from the mounted tree).  ``state.q`` is a numpy array
of shape (num_eqn, mx, my) in Fortran order, as PyClaw keeps it."""
from __future__ import annotations

import copy

import numpy as np

from .geometry import Domain, Patch


class State:
    def __init__(self, geom, num_eqn, num_aux=0):
        if isinstance(geom, Domain):
            self.patch = geom.patch
        elif isinstance(geom, Patch):
            self.patch = geom
        else:
            raise TypeError("State(domain_or_patch, num_eqn)")
        if num_aux:
            raise NotImplementedError("aux arrays are not supported by this backend")
        self.num_eqn = int(num_eqn)
        self.num_aux = 0
        self.problem_data = {}
        self.t = 0.0
        self.q = np.zeros([self.num_eqn] + self.patch.grid.num_cells, order="F")
        self.aux = None

    @property
    def grid(self):
        return self.patch.grid

    @property
    def num_dim(self):
        return self.patch.num_dim

    def __setattr__(self, name, value):
        if name == "q":
            value = np.asfortranarray(value, dtype=np.float64)
        object.__setattr__(self, name, value)


class Solution:
    """``Solution(state, domain)``; ``solution.t`` is the time of the state."""

    def __init__(self, state, domain=None):
        self.states = [state]
        self.domain = domain
        self.t = 0.0

    @property
    def state(self):
        return self.states[0]

    @property
    def q(self):
        return self.state.q

    @property
    def patch(self):
        return self.state.patch

    def copy(self):
        other = copy.copy(self)
        st = copy.copy(self.state)
        object.__setattr__(st, "q", self.state.q.copy(order="F"))
        st.problem_data = dict(self.state.problem_data)
        other.states = [st]
        return other
