"""Batches of independent classic 2D problems on one GPU.

``BatchSolver`` advances many problems of uneven grid sizes that share one
solver description (Riemann solver, boundary conditions, limiters, order,
transverse waves, precision, problem data).  Each problem keeps its own
time-step control (PyClaw's evolve_to_time rules: its own dt from its own
CFL, its own rejections and stop).  One ``advance(1)`` is one launch of the
batched step kernel, i.e. one attempted step of every unfinished problem;
``capture(n)`` records n of them in a CUDA graph.

Layout: the states of all problems are packed in two FP64 device buffers,
problem p at ``offsets[p]`` (in doubles, 32-byte aligned) in the
single-problem layout (num_eqn, mx, my) Fortran order.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .device import _stream_handle, make_solver_struct

CTRL_DTYPE = np.dtype([(name, {ctypes.c_double: "<f8", ctypes.c_int: "<i4",
                               ctypes.c_uint: "<u4"}.get(t, None) or ("<u8", (2,)))
                       for name, t in _lib.GclawCtrl._fields_])
assert CTRL_DTYPE.itemsize == _lib.CTRL_BYTES


class BatchSolver:
    def __init__(self, rp_id, shapes, deltas, bc_lower, bc_upper, mthlim, problem_data, order=2,
                 transverse_waves=2, precision=_lib.PREC_FP32_BULK, device=None):
        """shapes: list of (mx, my); deltas: list of (dx, dy)."""
        if len(shapes) != len(deltas) or not shapes:
            raise ValueError("shapes and deltas must be non-empty lists of equal length")
        self.L = _lib.lib()
        m = ctypes.c_int()
        mw = ctypes.c_int()
        _lib.check(self.L.gclaw_rp_shape(int(rp_id), ctypes.byref(m), ctypes.byref(mw)))
        self.m = m.value
        self.nprob = len(shapes)
        self.shapes = [(int(a), int(b)) for a, b in shapes]
        self.device = torch.device(device or "cuda")
        # shared solver description (grid fields are per problem)
        self.s = make_solver_struct(rp_id, 2, 2, 1.0, 1.0, bc_lower, bc_upper, mthlim, order,
                                    transverse_waves, precision, problem_data)
        sizes = np.array([self.m * a * b for a, b in self.shapes], dtype=np.int64)
        padded = (sizes + 3) // 4 * 4
        self.offsets = np.concatenate([[0], np.cumsum(padded)[:-1]]).astype(np.int64)
        self.sizes = sizes
        self.total = int(padded.sum())
        probs = (_lib.GclawBatchProblem * self.nprob)()
        for p, ((mx, my), (dx, dy)) in enumerate(zip(self.shapes, deltas)):
            probs[p].mx, probs[p].my = mx, my
            probs[p].dx, probs[p].dy = float(dx), float(dy)
            probs[p].q_offset = int(self.offsets[p])
        self.q = [torch.zeros(self.total, dtype=torch.float64, device=self.device),
                  torch.zeros(self.total, dtype=torch.float64, device=self.device)]
        self.ctrls = torch.zeros(self.nprob * _lib.CTRL_BYTES, dtype=torch.uint8,
                                 device=self.device)
        nb = self.L.gclaw_batch_table_bytes(self.nprob)
        self.table = torch.zeros(nb, dtype=torch.uint8, device=self.device)
        tiles = ctypes.c_int()
        _lib.check(self.L.gclaw_batch_prepare(ctypes.byref(self.s), probs, self.nprob,
                                              ctypes.c_void_p(self.table.data_ptr()), nb,
                                              ctypes.byref(tiles), _stream_handle()),
                   "gclaw_batch_prepare")
        self.total_tiles = tiles.value
        self.cells = int(sum(a * b for a, b in self.shapes))

    # ---------------------------------------------------------------- data
    def pinned_host_buffer(self):
        """A pinned host array of the packed-state size (fill with pack())."""
        return torch.empty(self.total, dtype=torch.float64, pin_memory=True)

    def pack(self, host, p, q):
        """Write problem p's (num_eqn, mx, my) state into a packed host buffer."""
        o, n = int(self.offsets[p]), int(self.sizes[p])
        host.numpy()[o:o + n] = np.asfortranarray(q, dtype=np.float64).ravel(order="F")

    def upload(self, host):
        self.q[0].copy_(host, non_blocking=False)

    def download(self):
        """All problems' accepted states, as a list of (num_eqn, mx, my) arrays."""
        c = self.read_ctrls()
        h = [self.q[0].cpu().numpy(), self.q[1].cpu().numpy()]
        out = []
        for p, (mx, my) in enumerate(self.shapes):
            o, n = int(self.offsets[p]), int(self.sizes[p])
            buf = h[int(c["parity"][p])][o:o + n]
            out.append(np.asfortranarray(buf.reshape((self.m, mx, my), order="F")))
        return out

    # ---------------------------------------------------------------- control
    def ctrl_init(self, dt0, t=0.0, t_end=math.inf, cfl_max=1.0, cfl_desired=0.9, dt_max=1e99,
                  max_steps=10000, max_accepted=-1, dt_variable=True, stream=None):
        d = torch.as_tensor(np.asarray(dt0, dtype=np.float64), device=self.device)
        self._dt0 = d  # kept alive while the init kernel may still read it
        _lib.check(self.L.gclaw_batch_ctrl_init(
            ctypes.c_void_p(self.ctrls.data_ptr()), self.nprob, ctypes.c_void_p(d.data_ptr()),
            float(t), float(t_end), float(cfl_max), float(cfl_desired), float(dt_max),
            int(max_steps), int(max_accepted), 1 if dt_variable else 0, _stream_handle(stream)),
            "gclaw_batch_ctrl_init")

    def read_ctrls(self):
        host = self.ctrls.cpu().numpy()
        return np.frombuffer(host.tobytes(), dtype=CTRL_DTYPE)

    def advance(self, nlaunch, stream=None):
        _lib.check(self.L.gclaw_batch_advance(
            ctypes.byref(self.s), ctypes.c_void_p(self.table.data_ptr()), self.nprob,
            self.total_tiles, ctypes.c_void_p(self.q[0].data_ptr()),
            ctypes.c_void_p(self.q[1].data_ptr()), ctypes.c_void_p(self.ctrls.data_ptr()),
            int(nlaunch), _stream_handle(stream)), "gclaw_batch_advance")

    def capture(self, nlaunch):
        """A CUDA graph of nlaunch batched steps (replay with .replay())."""
        self.advance(0)  # one-time kernel set-up outside the capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.advance(nlaunch, stream=s)
        return g
