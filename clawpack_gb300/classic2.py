"""``step2`` with the calling convention of PyClaw's f2py module classic2.

PyClaw's ClawSolver2D.step_hyperbolic (upstream
pyclaw/src/pyclaw/classic/solver.py) calls

    q, cfl = self.fmod.step2(maxm, num_ghost, mx, my, qold, qbc, auxbc,
                             dx, dy, dt, method, mthlim, fwave, rpn2, rpt2)

with ``qold``/``qbc`` of shape (num_eqn, mx+2*num_ghost, my+2*num_ghost) in
Fortran order, ``auxbc`` the ghost-filled aux array (num_aux, mx+4, my+4)
(or empty), ``method`` the 7-entry integer array (method[1] = order,
method[2] = transverse_waves, method[5] = mcapa = state.index_capa + 1,
method[6] = num_aux), ``mthlim`` the limiter id per wave, ``fwave`` whether
the solver returns f-waves, and ``rpn2``/``rpt2`` the Riemann solver
module.  Pointing ``self.fmod`` at this
module runs the step on the GPU through ``gclaw_step2``: the arrays may be
numpy (copied to and from the device each call, as the reference passes
them) or CUDA torch tensors of shape (my+4, mx+4, num_eqn) that stay on the
device.  Physical parameters come from the solver module's ``cparam``
namespace, which PyClaw fills from ``state.problem_data``.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .device import make_solver_struct

_ws = {}


def _workspace(device):
    key = str(device)
    if key not in _ws:
        _ws[key] = torch.zeros(256, dtype=torch.uint8, device=device)
    return _ws[key]


def _problem_data(rp):
    c = rp.cparam
    if rp.rp_id == _lib.RP_ACOUSTICS_2D:
        rho, bulk = float(c.rho), float(c.bulk)
        cc = float(getattr(c, "cc", math.sqrt(bulk / rho)))
        zz = float(getattr(c, "zz", rho * cc))
        return [rho, bulk, cc, zz]
    if rp.rp_id in (_lib.RP_SHALLOW_ROE_WITH_EFIX_2D, _lib.RP_SHALLOW_BATHYMETRY_FWAVE_2D):
        return [float(c.grav)]
    if rp.rp_id == _lib.RP_VC_ACOUSTICS_2D:
        return []
    return [float(c.gamma), 1.0 if getattr(c, "efix", True) else 0.0]


def _device_array(a):
    """A ghost-filled (n, mx+4, my+4) host array as the device layout
    (my+4, mx+4, n), or a CUDA tensor already in that layout."""
    if isinstance(a, torch.Tensor):
        return a
    return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a, dtype=np.float64).T)).cuda()


def step2(maxm, num_ghost, mx, my, qold, qnew, aux, dx, dy, dt, method, mthlim, fwave, rpn2,
          rpt2, bc_lower=(1, 1), bc_upper=(1, 1), precision=_lib.PREC_FP64):
    """One unsplit step; returns (qnew, cfl) like the f2py routine."""
    if num_ghost != 2:
        raise ValueError("num_ghost must be 2")
    if bool(fwave) != bool(getattr(rpn2, "fwave", False)):
        raise ValueError(f"{rpn2.name} needs fwave = {bool(getattr(rpn2, 'fwave', False))}")
    order, tw = int(method[1]), int(method[2])
    mcapa = int(method[5]) if len(method) > 5 else 0
    if tw < 0:
        raise NotImplementedError("dimensional splitting is not supported")
    has_aux = aux is not None and (aux.numel() if isinstance(aux, torch.Tensor) else np.size(aux))
    # The ghost cells are already filled; bc ids only have to pass validation.
    s = make_solver_struct(rpn2.rp_id, mx, my, dx, dy, bc_lower, bc_upper, list(mthlim), order,
                           tw, precision, _problem_data(rpn2), capa=mcapa)
    d_aux = None
    if has_aux:
        d_aux = _device_array(aux)  # stream-ordered: safe to drop after the launch
        s.aux = d_aux.data_ptr()
    L = _lib.lib()
    cfl = ctypes.c_double()
    if isinstance(qold, torch.Tensor):
        d_old, d_new = qold, qnew
        stream = torch.cuda.current_stream(d_old.device)
        ws = _workspace(d_old.device)
    else:
        d_old = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(qold).T)).cuda()
        d_new = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(qnew).T)).cuda()
        stream = torch.cuda.current_stream()
        ws = _workspace(d_old.device)
    rc = L.gclaw_step2(ctypes.byref(s), ctypes.c_void_p(d_old.data_ptr()),
                       ctypes.c_void_p(d_new.data_ptr()), float(dt), ctypes.c_void_p(ws.data_ptr()),
                       ctypes.byref(cfl), ctypes.c_void_p(stream.cuda_stream))
    _lib.check(rc, "gclaw_step2")
    if isinstance(qold, torch.Tensor):
        return qnew, cfl.value
    out = np.asfortranarray(d_new.cpu().numpy().T)
    if isinstance(qnew, np.ndarray) and qnew.flags.f_contiguous and qnew.shape == out.shape:
        qnew[...] = out
        return qnew, cfl.value
    return out, cfl.value
