"""Controller.run() with PyClaw's output-time loop (upstream
pyclaw/src/pyclaw/controller.py; absent from the mounted tree).

output_style 1: frames at num_output_times equally spaced times from the
initial time to tfinal; output_style 2: the times in ``out_times``.  Frames are
kept in memory (``keep_copy``); writing them to disk is not part of this
package.
"""
from __future__ import annotations

import logging

import numpy as np


class Controller:
    def __init__(self):
        self.solution = None
        self.solver = None
        self.tfinal = 1.0
        self.num_output_times = 10
        self.output_style = 1
        self.out_times = None
        self.keep_copy = True
        self.output_format = None
        self.frames = []
        self.logger = logging.getLogger("pyclaw.controller")

    def run(self):
        if self.solution is None or self.solver is None:
            raise ValueError("Controller.solution and Controller.solver must be set")
        t0 = self.solution.t
        if self.output_style == 1:
            times = np.linspace(t0, self.tfinal, self.num_output_times + 1)
        elif self.output_style == 2:
            times = np.asarray(self.out_times, dtype=float)
        else:
            raise NotImplementedError("output_style must be 1 or 2")
        self.solver.setup(self.solution)
        self.frames = []
        if self.keep_copy:
            self.frames.append(self.solution.copy())
        status = self.solver.status
        for k, t_out in enumerate(times[1:], start=1):
            status = self.solver.evolve_to_time(self.solution, t_out)
            if self.keep_copy:
                self.frames.append(self.solution.copy())
            self.logger.info("Solution %d computed for time t=%f", k, self.solution.t)
        return status
