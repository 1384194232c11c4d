"""Gradients through time stepping: a torch.autograd.Function around the
classic 2D step and its hand-written adjoint kernel (gclaw_adjoint_step).

``evolve_gauges(q0, problem, dts, gauges, checkpoint_every)`` advances q0
(num_eqn, mx, my) through len(dts) steps with the given dt sequence and
returns the depth / first component at the gauge cells after every step,
shape (N, G).  Its backward computes d loss / d q0 by the discrete adjoint:
states are checkpointed every ``checkpoint_every`` steps in the forward pass
(about sqrt(N) checkpoints), each segment is recomputed from its checkpoint
in the backward pass, and the adjoint steps run in reverse through it.  The
dt sequence is an input (chosen by ``record_dts`` with PyClaw's CFL rule on
the undisturbed run) and is held fixed, so the gradient is that of the
discrete map actually run, limiter and entropy-fix branches included.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .device import DeviceProblem, _stream_handle


def _to_dev(q):
    """(m, mx, my) tensor -> contiguous device layout (my, mx, m)."""
    return q.permute(2, 1, 0).contiguous()


def _from_dev(d):
    return d.permute(2, 1, 0)


class _Stepper:
    """Explicit-dt steps and adjoint steps on device tensors (my, mx, m)."""

    def __init__(self, solver_struct, device):
        self.s = solver_struct
        self.L = _lib.lib()
        self.ws = torch.zeros(256, dtype=torch.uint8, device=device)

    def step(self, q, dt, out=None):
        out = torch.empty_like(q) if out is None else out
        _lib.check(self.L.gclaw_step(ctypes.byref(self.s), ctypes.c_void_p(q.data_ptr()),
                                     ctypes.c_void_p(out.data_ptr()), float(dt),
                                     ctypes.c_void_p(self.ws.data_ptr()), _stream_handle()),
                   "gclaw_step")
        return out

    def adjoint(self, q, lam, dt):
        out = torch.empty_like(lam)
        _lib.check(self.L.gclaw_adjoint_step(ctypes.byref(self.s), ctypes.c_void_p(q.data_ptr()),
                                             ctypes.c_void_p(lam.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()), float(dt),
                                             _stream_handle()), "gclaw_adjoint_step")
        return out


class EvolveGauges(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q0, solver_struct, dts, gauges, checkpoint_every):
        dev = q0.device
        st = _Stepper(solver_struct, dev)
        gy, gx = gauges[:, 1], gauges[:, 0]
        q = _to_dev(q0.detach())
        n = len(dts)
        out = torch.empty((n, gauges.shape[0]), dtype=torch.float64, device=dev)
        ckpts = []
        for k in range(n):
            if k % checkpoint_every == 0:
                ckpts.append(q.clone())
            q = st.step(q, dts[k])
            out[k] = q[gy, gx, 0]
        ctx.st, ctx.dts, ctx.ckpts, ctx.K = st, list(dts), ckpts, checkpoint_every
        ctx.gauges = gauges
        return out

    @staticmethod
    def backward(ctx, gout):
        st, dts, K = ctx.st, ctx.dts, ctx.K
        gy, gx = ctx.gauges[:, 1], ctx.gauges[:, 0]
        n = len(dts)
        lam = torch.zeros_like(ctx.ckpts[0])
        comp0 = torch.zeros_like(gy)
        for seg in range(len(ctx.ckpts) - 1, -1, -1):
            start, stop = seg * K, min((seg + 1) * K, n)
            states = [ctx.ckpts[seg]]
            for k in range(start, stop - 1):
                states.append(st.step(states[-1], dts[k]))
            for k in range(stop - 1, start - 1, -1):
                # accumulate: several gauges may sit in one cell
                lam.index_put_((gy, gx, comp0), gout[k], accumulate=True)
                lam = st.adjoint(states[k - start], lam, dts[k])
        return _from_dev(lam), None, None, None, None


def evolve_gauges(q0, solver_struct, dts, gauges, checkpoint_every=23):
    """Gauge series (N, G) of component 0 after each of the N steps; q0 is a
    CUDA float64 tensor (num_eqn, mx, my); gauges an int64 tensor (G, 2) of
    (i, j) cell indices on q0's device."""
    return EvolveGauges.apply(q0, solver_struct, dts, gauges, checkpoint_every)


def evolve_fixed(q0, solver_struct, dts):
    """State after len(dts) steps of the given sizes (no gradient)."""
    st = _Stepper(solver_struct, q0.device)
    q = _to_dev(q0)
    for dt in dts:
        q = st.step(q, dt)
    return _from_dev(q)


def gauge_series(q0, solver_struct, dts, gauges):
    """Gauge series of a run with fixed dts (no gradient)."""
    st = _Stepper(solver_struct, q0.device)
    gy, gx = gauges[:, 1], gauges[:, 0]
    q = _to_dev(q0.detach())
    out = torch.empty((len(dts), gauges.shape[0]), dtype=torch.float64, device=q0.device)
    for k, dt in enumerate(dts):
        q = st.step(q, dt)
        out[k] = q[gy, gx, 0]
    return out


def record_dts(q0, solver_struct, nsteps, dt0, cfl_desired=0.9, cfl_max=1.0):
    """The accepted dt sequence of an nsteps run from q0 under PyClaw's rules
    (reject when cfl > cfl_max, dt = dt cfl_desired / cfl)."""
    dp = DeviceProblem(solver_struct, device=q0.device)
    dp.upload(q0.detach().cpu().numpy())
    dts, dt, src = [], float(dt0), 0
    while len(dts) < nsteps:
        dp.step(dt, src=src)
        c = dp.read_ctrl()
        _lib.check(c.status, "record_dts")
        if c.cfl <= cfl_max:
            dts.append(dt)
            src ^= 1
        dt = dt * cfl_desired / c.cfl if c.cfl > 0 else dt
    return dts
