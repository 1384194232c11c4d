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
        self.num_eqn = int(num_eqn)
        self.num_aux = int(num_aux)
        # aux field holding the capacity function (-1: none), as in PyClaw
        self.index_capa = -1
        self.problem_data = {}
        self.t = 0.0
        self.q = np.zeros([self.num_eqn] + self.patch.grid.num_cells, order="F")
        self.aux = (np.zeros([self.num_aux] + self.patch.grid.num_cells, order="F")
                    if self.num_aux else None)

    @property
    def grid(self):
        return self.patch.grid

    @property
    def num_dim(self):
        return self.patch.num_dim

    def __setattr__(self, name, value):
        if name == "q" or (name == "aux" and value is not None):
            value = np.asfortranarray(value, dtype=np.float64)
        object.__setattr__(self, name, value)


class Solution:
    """``Solution(state, domain)``, or ``Solution(frame, path=..., file_format=...,
    file_prefix=..., read_aux=...)`` to load an output frame; ``solution.t``
    is the time of the state."""

    def __init__(self, state, domain=None, path="./_output", file_format="ascii",
                 file_prefix=None, read_aux=False):
        self.states = []
        self.domain = domain
        self.t = 0.0
        if isinstance(state, (int, np.integer)):
            self.read(int(state), path, file_format, file_prefix, read_aux)
        else:
            self.states = [state]

    def write(self, frame, path="./", file_format="ascii", file_prefix=None, write_aux=False,
              options=None, write_p=False):
        """Write this solution as output frame ``frame`` (formats 'ascii' and
        'binary', see clawpack_gb300.pyclaw.fileio)."""
        from . import fileio

        fileio.module(file_format).write(self, frame, path, file_prefix or "fort", write_aux,
                                         options or {}, write_p)

    def read(self, frame, path="./_output", file_format="ascii", file_prefix=None,
             read_aux=False, options=None):
        """Replace this solution's state by output frame ``frame``."""
        from . import fileio

        return fileio.module(file_format).read(self, frame, path, file_prefix or "fort",
                                               read_aux, options or {})

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
