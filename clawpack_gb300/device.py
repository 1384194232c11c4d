"""Device-resident problem state for libgclaw.so: two FP64 state buffers, a
gclaw_ctrl block, and thin wrappers over the C ABI.

PyTorch provides device memory and the stream; every kernel is libgclaw's.
The state buffers hold q as PyClaw lays it out, (num_eqn, mx, my) in Fortran
order, which is a C-contiguous torch tensor of shape (my, mx, num_eqn).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def _stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def make_solver_struct(rp_id, mx, my, dx, dy, bc_lower, bc_upper, mthlim, order, tw,
                       precision, problem_data, aux_bc_lower=(1, 1), aux_bc_upper=(1, 1),
                       capa=0):
    s = _lib.GclawSolver()
    s.rp = int(rp_id)
    s.mx, s.my = int(mx), int(my)
    s.dx, s.dy = float(dx), float(dy)
    for d in range(2):
        s.bc_lower[d] = int(bc_lower[d])
        s.bc_upper[d] = int(bc_upper[d])
    lim = list(mthlim) + [0] * (_lib.MAX_WAVES - len(mthlim))
    for p in range(_lib.MAX_WAVES):
        s.mthlim[p] = int(lim[p])
    s.order = int(order)
    s.transverse_waves = int(tw)
    s.precision = int(precision)
    pd = list(problem_data) + [0.0] * (8 - len(problem_data))
    for i in range(8):
        s.problem_data[i] = float(pd[i])
    for d in range(2):
        s.aux_bc_lower[d] = int(aux_bc_lower[d])
        s.aux_bc_upper[d] = int(aux_bc_upper[d])
    s.capa = int(capa)
    return s


class DeviceProblem:
    """Two state buffers + control block on one CUDA device.  With
    ``split=True`` steps are dimensionally split (x-sweep, then y-sweep) and a
    third buffer holds the state between the sweeps."""

    def __init__(self, solver_struct, device=None, strict=False, split=False, aux=None):
        self.s = solver_struct
        self.L = L = _lib.lib(strict)
        self.device = torch.device(device or "cuda")
        self.aux = None
        if aux is not None:
            self.set_aux(aux)
        _lib.check(L.gclaw_check(ctypes.byref(self.s)), "gclaw_check")
        m = ctypes.c_int()
        mw = ctypes.c_int()
        _lib.check(L.gclaw_rp_shape(self.s.rp, ctypes.byref(m), ctypes.byref(mw)))
        self.m, self.mw = m.value, mw.value
        self.mx, self.my = self.s.mx, self.s.my
        shape = (self.my, self.mx, self.m)
        self.q = [torch.empty(shape, dtype=torch.float64, device=self.device),
                  torch.empty(shape, dtype=torch.float64, device=self.device)]
        self.split = bool(split)
        self.qtmp = (torch.empty(shape, dtype=torch.float64, device=self.device)
                     if self.split else None)
        self.ctrl = torch.zeros(256, dtype=torch.uint8, device=self.device)
        self._ctrl_host = torch.empty(256, dtype=torch.uint8, pin_memory=True)
        self.ctrl_init(0.0, 1.0, 0.0)

    def set_aux(self, aux):
        """Copy a host (num_aux, mx, my) aux array to the device and point the
        solver description at it (solvers with an aux array)."""
        af = np.asfortranarray(aux, dtype=np.float64)
        if af.shape[1:] != (self.s.mx, self.s.my):
            raise ValueError(f"aux has shape {af.shape}, expected (num_aux, {self.s.mx}, "
                             f"{self.s.my})")
        t = torch.from_numpy(af.T.copy()).to(self.device)
        self.aux = t  # keeps the device array alive while the struct points at it
        self.s.aux = t.data_ptr()

    # -- host <-> device ---------------------------------------------------
    def upload(self, q, buf=0):
        """Copy a host (num_eqn, mx, my) array into state buffer ``buf``."""
        qf = np.asfortranarray(q, dtype=np.float64)
        if qf.shape != (self.m, self.mx, self.my):
            raise ValueError(f"q has shape {qf.shape}, expected {(self.m, self.mx, self.my)}")
        self.q[buf].copy_(torch.from_numpy(qf.T))

    def download(self, buf=0):
        """State buffer ``buf`` as a host (num_eqn, mx, my) Fortran-ordered array."""
        return np.asfortranarray(self.q[buf].cpu().numpy().T)

    # -- control block -------------------------------------------------------
    def ctrl_init(self, t, dt, t_end, cfl_max=1.0, cfl_desired=0.9, dt_max=1e99,
                  max_steps=10000, max_accepted=-1, dt_variable=True, stream=None):
        _lib.check(self.L.gclaw_ctrl_init(
            ctypes.c_void_p(self.ctrl.data_ptr()), float(t), float(dt), float(t_end),
            float(cfl_max), float(cfl_desired), float(dt_max), int(max_steps),
            int(max_accepted), 1 if dt_variable else 0, _stream_handle(stream)), "gclaw_ctrl_init")

    def read_ctrl(self, stream=None):
        """Synchronise the stream and return a host copy of the gclaw_ctrl."""
        self._ctrl_host.copy_(self.ctrl, non_blocking=True)
        (stream or torch.cuda.current_stream()).synchronize()
        c = _lib.GclawCtrl()
        ctypes.memmove(ctypes.addressof(c), self._ctrl_host.data_ptr(), _lib.CTRL_BYTES)
        return c

    # -- stepping ------------------------------------------------------------
    def advance(self, nlaunch, stream=None):
        """Enqueue ``nlaunch`` controlled steps (no synchronisation)."""
        if self.split:
            _lib.check(self.L.gclaw_advance_split(
                ctypes.byref(self.s), ctypes.c_void_p(self.q[0].data_ptr()),
                ctypes.c_void_p(self.q[1].data_ptr()), ctypes.c_void_p(self.qtmp.data_ptr()),
                ctypes.c_void_p(self.ctrl.data_ptr()), int(nlaunch), _stream_handle(stream)),
                "gclaw_advance_split")
            return
        _lib.check(self.L.gclaw_advance(
            ctypes.byref(self.s), ctypes.c_void_p(self.q[0].data_ptr()),
            ctypes.c_void_p(self.q[1].data_ptr()), ctypes.c_void_p(self.ctrl.data_ptr()),
            int(nlaunch), _stream_handle(stream)), "gclaw_advance")

    def step(self, dt, src=0, stream=None):
        """One step with explicit dt from buffer ``src`` into ``1 - src``; the
        Courant number is left in the control block (see ``read_ctrl``)."""
        if self.split:
            _lib.check(self.L.gclaw_step_split(
                ctypes.byref(self.s), ctypes.c_void_p(self.q[src].data_ptr()),
                ctypes.c_void_p(self.q[1 - src].data_ptr()),
                ctypes.c_void_p(self.qtmp.data_ptr()), float(dt),
                ctypes.c_void_p(self.ctrl.data_ptr()), _stream_handle(stream)),
                "gclaw_step_split")
            return
        _lib.check(self.L.gclaw_step(
            ctypes.byref(self.s), ctypes.c_void_p(self.q[src].data_ptr()),
            ctypes.c_void_p(self.q[1 - src].data_ptr()), float(dt),
            ctypes.c_void_p(self.ctrl.data_ptr()), _stream_handle(stream)), "gclaw_step")

    def evolve(self, t, dt, t_end, *, cfl_max=1.0, cfl_desired=0.9, dt_max=1e99,
               max_steps=10000, max_accepted=-1, dt_variable=True, batch=32, stream=None):
        """Device-controlled evolve of buffer 0 (already uploaded); returns the
        final control block.  The accepted state is in buffer ``ctrl.parity``."""
        self.ctrl_init(t, dt, t_end, cfl_max, cfl_desired, dt_max, max_steps, max_accepted,
                       dt_variable, stream)
        while True:
            self.advance(batch, stream)
            c = self.read_ctrl(stream)
            if c.done:
                return c


def make_solver3_struct(rp_id, mx, my, mz, dx, dy, dz, bc_lower, bc_upper, mthlim, order, tw,
                        precision, problem_data):
    """The gclaw3_solver C struct (include/gclaw3.h)."""
    s = _lib.GclawSolver3()
    s.rp = int(rp_id)
    s.mx, s.my, s.mz = int(mx), int(my), int(mz)
    s.dx, s.dy, s.dz = float(dx), float(dy), float(dz)
    for d in range(3):
        s.bc_lower[d] = int(bc_lower[d])
        s.bc_upper[d] = int(bc_upper[d])
    lim = list(mthlim) + [0] * (_lib.MAX_WAVES - len(mthlim))
    for p in range(_lib.MAX_WAVES):
        s.mthlim[p] = int(lim[p])
    s.order = int(order)
    s.transverse_waves = int(tw)
    s.precision = int(precision)
    pd = list(problem_data) + [0.0] * (8 - len(problem_data))
    for i in range(8):
        s.problem_data[i] = float(pd[i])
    return s


class DeviceProblem3(DeviceProblem):
    """The 3D counterpart: two (num_eqn, mx, my, mz) state buffers, the step's
    workspace and a control block on one CUDA device (gclaw3_step /
    gclaw3_advance); time-step control as in 2D."""

    def __init__(self, solver_struct, device=None, strict=False, split=False):
        self.s = solver_struct
        self.L = L = _lib.lib(strict)
        self.device = torch.device(device or "cuda")
        self.split = bool(split)
        self.aux = None
        _lib.check(L.gclaw3_check(ctypes.byref(self.s)), "gclaw3_check")
        m, mw = ctypes.c_int(), ctypes.c_int()
        _lib.check(L.gclaw3_rp_shape(self.s.rp, ctypes.byref(m), ctypes.byref(mw)))
        self.m, self.mw = m.value, mw.value
        self.mx, self.my, self.mz = self.s.mx, self.s.my, self.s.mz
        shape = (self.mz, self.my, self.mx, self.m)
        self.q = [torch.empty(shape, dtype=torch.float64, device=self.device),
                  torch.empty(shape, dtype=torch.float64, device=self.device)]
        self.qtmp = (torch.empty(shape, dtype=torch.float64, device=self.device)
                     if self.split else None)
        # split sweeps keep no edge records
        nbytes = 0 if self.split else L.gclaw3_workspace_bytes(ctypes.byref(self.s))
        self.ws = torch.empty(int(nbytes), dtype=torch.uint8, device=self.device)
        self.ctrl = torch.zeros(256, dtype=torch.uint8, device=self.device)
        self._ctrl_host = torch.empty(256, dtype=torch.uint8, pin_memory=True)
        self.ctrl_init(0.0, 1.0, 0.0)

    def upload(self, q, buf=0):
        """Copy a host (num_eqn, mx, my, mz) array into state buffer ``buf``."""
        qf = np.asfortranarray(q, dtype=np.float64)
        if qf.shape != (self.m, self.mx, self.my, self.mz):
            raise ValueError(f"q has shape {qf.shape}, expected "
                             f"{(self.m, self.mx, self.my, self.mz)}")
        self.q[buf].copy_(torch.from_numpy(qf.T))

    def download(self, buf=0):
        return np.asfortranarray(self.q[buf].cpu().numpy().T)

    def advance(self, nlaunch, stream=None):
        if self.split:
            _lib.check(self.L.gclaw3_advance_split(
                ctypes.byref(self.s), ctypes.c_void_p(self.q[0].data_ptr()),
                ctypes.c_void_p(self.q[1].data_ptr()), ctypes.c_void_p(self.qtmp.data_ptr()),
                ctypes.c_void_p(self.ws.data_ptr()), ctypes.c_void_p(self.ctrl.data_ptr()),
                int(nlaunch), _stream_handle(stream)), "gclaw3_advance_split")
            return
        _lib.check(self.L.gclaw3_advance(
            ctypes.byref(self.s), ctypes.c_void_p(self.q[0].data_ptr()),
            ctypes.c_void_p(self.q[1].data_ptr()), ctypes.c_void_p(self.ws.data_ptr()),
            ctypes.c_void_p(self.ctrl.data_ptr()), int(nlaunch), _stream_handle(stream)),
            "gclaw3_advance")

    def step(self, dt, src=0, stream=None):
        if self.split:
            _lib.check(self.L.gclaw3_step_split(
                ctypes.byref(self.s), ctypes.c_void_p(self.q[src].data_ptr()),
                ctypes.c_void_p(self.q[1 - src].data_ptr()),
                ctypes.c_void_p(self.qtmp.data_ptr()), float(dt),
                ctypes.c_void_p(self.ws.data_ptr()), ctypes.c_void_p(self.ctrl.data_ptr()),
                _stream_handle(stream)), "gclaw3_step_split")
            return
        _lib.check(self.L.gclaw3_step(
            ctypes.byref(self.s), ctypes.c_void_p(self.q[src].data_ptr()),
            ctypes.c_void_p(self.q[1 - src].data_ptr()), float(dt),
            ctypes.c_void_p(self.ws.data_ptr()), ctypes.c_void_p(self.ctrl.data_ptr()),
            _stream_handle(stream)), "gclaw3_step")
