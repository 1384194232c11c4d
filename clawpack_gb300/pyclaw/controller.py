"""Controller.run() with PyClaw's output-time loop (upstream
pyclaw/src/pyclaw/controller.py; absent from the mounted tree).

output_style 1: frames at num_output_times equally spaced times from the
initial time to tfinal; output_style 2: the times in ``out_times``.  Frames are
kept in memory (``keep_copy``) and, when ``output_format`` is 'ascii' or
'binary', written to ``outdir`` as ``<output_file_prefix>.t/q/bNNNN`` (frame 0
is the initial state).  ``output_format`` defaults to None (no files), since
ascii frames of large grids take far longer to write than to compute.
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
        self.outdir = "./_output"
        self.output_file_prefix = None
        self.output_options = {}
        # aux arrays in the frame files: with frame 0 only, or with every frame
        self.write_aux_init = False
        self.write_aux_always = False
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
        self._output(0)
        status = self.solver.status
        for k, t_out in enumerate(times[1:], start=1):
            status = self.solver.evolve_to_time(self.solution, t_out)
            self._output(k)
            self.logger.info("Solution %d computed for time t=%f", k, self.solution.t)
        return status

    def _output(self, frame):
        if self.keep_copy:
            self.frames.append(self.solution.copy())
        if self.output_format is not None:
            aux = self.write_aux_always or (self.write_aux_init and frame == 0)
            self.solution.write(frame, self.outdir, self.output_format, self.output_file_prefix,
                                write_aux=aux, options=self.output_options)
