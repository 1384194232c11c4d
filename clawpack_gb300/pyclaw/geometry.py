"""Grid objects with PyClaw's names: Dimension, Patch/Grid, Domain
(upstream pyclaw/src/pyclaw/geometry.py; absent from the mounted tree)."""
from __future__ import annotations

import numpy as np


class Dimension:
    """One coordinate direction: ``Dimension(lower, upper, num_cells, name)``."""

    def __init__(self, lower, upper, num_cells, name="x"):
        if upper <= lower:
            raise ValueError("upper must exceed lower")
        if int(num_cells) < 1:
            raise ValueError("num_cells must be positive")
        self.lower = float(lower)
        self.upper = float(upper)
        self.num_cells = int(num_cells)
        self.name = name

    @property
    def delta(self):
        return (self.upper - self.lower) / self.num_cells

    @property
    def centers(self):
        return self.lower + (np.arange(self.num_cells) + 0.5) * self.delta

    @property
    def nodes(self):
        return self.lower + np.arange(self.num_cells + 1) * self.delta

    def __repr__(self):
        return f"Dimension({self.lower}, {self.upper}, {self.num_cells}, name={self.name!r})"


class Grid:
    """Cartesian grid of a patch; ``p_centers``/``c_centers`` are the
    physical/computational cell centres as an ``indexing='ij'`` mesh."""

    def __init__(self, dimensions):
        self.dimensions = list(dimensions)
        self.num_dim = len(self.dimensions)

    @property
    def num_cells(self):
        return [d.num_cells for d in self.dimensions]

    @property
    def delta(self):
        return [d.delta for d in self.dimensions]

    @property
    def lower(self):
        return [d.lower for d in self.dimensions]

    @property
    def upper(self):
        return [d.upper for d in self.dimensions]

    @property
    def c_centers(self):
        return np.meshgrid(*[d.centers for d in self.dimensions], indexing="ij")

    @property
    def p_centers(self):
        return self.c_centers

    def __getattr__(self, name):
        for d in self.__dict__.get("dimensions", []):
            if d.name == name:
                return d
        raise AttributeError(name)


class Patch:
    def __init__(self, dimensions):
        self.dimensions = list(dimensions)
        self.grid = Grid(self.dimensions)
        self.num_dim = len(self.dimensions)


class Domain:
    """``Domain([dim_x, dim_y])`` or ``Domain(lower, upper, num_cells)``."""

    def __init__(self, *args):
        if len(args) == 1:
            dims = args[0]
            if isinstance(dims, Dimension):
                dims = [dims]
        elif len(args) == 3:
            lower, upper, n = args
            names = ["x", "y", "z"]
            dims = [Dimension(lo, up, k, name=names[i])
                    for i, (lo, up, k) in enumerate(zip(lower, upper, n))]
        else:
            raise TypeError("Domain(dimensions) or Domain(lower, upper, num_cells)")
        self.patch = Patch(dims)
        self.patches = [self.patch]
        self.grid = self.patch.grid
        self.num_dim = self.patch.num_dim
