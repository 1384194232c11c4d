"""The host-buffer entry points (gclaw_step_host, gclaw_evolve_host): the
reference's calling pattern, numpy state in and out of every call.

gclaw_step_host takes raw caller memory as its workspace, so it is tested
with a workspace full of 0xFF bytes and must still reproduce the oracle bit
for bit (strict build) on every call; gclaw_evolve_host must give the same
state and control block as the device-resident evolve."""
import ctypes
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import PD, SHAPES, random_state

pytestmark = pytest.mark.gpu


def aligned_workspace(nbytes, fill):
    buf = torch.full((nbytes + 256,), fill, dtype=torch.uint8, device="cuda")
    base = (buf.data_ptr() + 255) // 256 * 256
    return buf, base


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_step_host_with_dirty_workspace_is_bitwise(cuda, oracle, rp):
    mx, my = 45, 38
    rng = np.random.default_rng(11 + rp)
    q = np.asfortranarray(random_state(rp, mx, my, rng))
    dx, dy = 1.0 / mx, 1.1 / my
    dt = 0.05 * min(dx, dy)
    bcl, bcu = [3, 1], [1, 3]
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [4] * SHAPES[rp][1], 2, 2, 0, PD[rp])
    L = _lib.lib(strict=True)
    nb = L.gclaw_step_workspace_bytes(ctypes.byref(s))
    buf, base = aligned_workspace(nb, 0xFF)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    qcur = q
    for _ in range(3):  # the workspace is reused without clearing by the caller
        qo, cflo, rc = oracle.step(rp, PD[rp], qcur, dx, dy, dt, bcl, bcu, 2, 2, [4] * 4)
        assert rc == 0
        out = np.empty_like(qcur, order="F")
        cfl = ctypes.c_double(-1.0)
        status = L.gclaw_step_host(ctypes.byref(s), ptr(qcur), ptr(out), dt, ctypes.c_void_p(base),
                                   nb, ctypes.byref(cfl), stream)
        assert status == 0
        assert np.array_equal(out, qo)
        assert cfl.value == cflo
        qcur = out


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("bcl,bcu", [([3, 1], [1, 3]), ([1, 2], [1, 2])])
def test_step_host_bands_are_bitwise(cuda, oracle, rp, bcl, bcu):
    """A grid tall enough for the band-by-band host step (FP64 tiles, copies
    overlapping the bands): the same bits as the oracle in the strict build,
    with a periodic y boundary (one launch) as well."""
    mx, my = 70, 300
    rng = np.random.default_rng(21 + rp)
    q = np.asfortranarray(random_state(rp, mx, my, rng))
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [4] * SHAPES[rp][1], 2, 2, 0, PD[rp])
    L = _lib.lib(strict=True)
    nb = L.gclaw_step_workspace_bytes(ctypes.byref(s))
    buf, base = aligned_workspace(nb, 0xFF)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, bcl, bcu, 2, 2, [4] * 4)
    out = np.empty_like(q, order="F")
    cfl = ctypes.c_double(-1.0)
    status = L.gclaw_step_host(ctypes.byref(s), ptr(q), ptr(out), dt, ctypes.c_void_p(base), nb,
                               ctypes.byref(cfl), stream)
    assert status == 0
    assert np.array_equal(out, qo)
    assert cfl.value == cflo


def test_evolve_host_matches_device_evolve(cuda):
    rp, mx, my = 2, 64, 40
    X, Y = np.meshgrid((np.arange(mx) + 0.5) / mx, (np.arange(my) + 0.5) / my, indexing="ij")
    q = np.zeros((3, mx, my), order="F")
    q[0] = 1.0 + 0.4 * np.exp(-40.0 * ((X - 0.4) ** 2 + (Y - 0.6) ** 2))  # a hump at rest
    dx, dy = 1.0 / mx, 1.0 / my
    s = make_solver_struct(rp, mx, my, dx, dy, [3, 3], [3, 3], [4] * 3, 2, 2, 0, PD[rp])
    dt0, tend = 0.5 * dx, 0.08
    dev = DeviceProblem(s)
    dev.upload(q)
    c = dev.evolve(0.0, dt0, tend, max_steps=1000)
    assert c.status == 0 and c.numsteps > 5
    ref = dev.download(c.parity)
    L = _lib.lib()
    nb = L.gclaw_evolve_workspace_bytes(ctypes.byref(s))
    buf, base = aligned_workspace(nb, 0x5A)
    out = np.empty_like(q, order="F")
    ctrl = _lib.GclawCtrl()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = L.gclaw_evolve_host(ctypes.byref(s), ptr(q), ptr(out), 0.0, dt0, tend, -1, 1.0, 0.9,
                                 1e99, 1000, ctypes.c_void_p(base), nb, 32, ctypes.byref(ctrl),
                                 stream)
    assert status == 0
    assert ctrl.done == 1 and ctrl.status == 0
    assert math.isclose(ctrl.t, tend, rel_tol=0, abs_tol=1e-14)
    assert (ctrl.t, ctrl.numsteps, ctrl.attempts) == (c.t, c.numsteps, c.attempts)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("rp,prec", [(2, 0), (3, 0), (2, 1)])
def test_step_host_pinned_arrays_zero_copy(cuda, oracle, rp, prec):
    """Pinned host arrays: the step reads and writes them directly; the same
    bits as the oracle (strict build, FP64) or as the pageable path (FP32)."""
    mx, my = 90, 140
    rng = np.random.default_rng(31 + rp)
    q = np.asfortranarray(random_state(rp, mx, my, rng))
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    bcl, bcu = [3, 1], [1, 3]
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [4] * SHAPES[rp][1], 2, 2, prec,
                           PD[rp])
    L = _lib.lib(strict=prec == 0)
    nb = L.gclaw_step_workspace_bytes(ctypes.byref(s))
    buf, base = aligned_workspace(nb, 0xFF)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    pin_in = torch.from_numpy(np.ascontiguousarray(q.T)).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    cfl = ctypes.c_double(-1.0)
    st = L.gclaw_step_host(ctypes.byref(s), ctypes.c_void_p(pin_in.data_ptr()),
                           ctypes.c_void_p(pin_out.data_ptr()), dt, ctypes.c_void_p(base), nb,
                           ctypes.byref(cfl), stream)
    assert st == 0
    out = np.asfortranarray(pin_out.numpy().T)
    if prec == 0:
        qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, bcl, bcu, 2, 2, [4] * 4)
        assert np.array_equal(out, qo)
        assert cfl.value == cflo
    else:
        ref = np.empty_like(q, order="F")
        cfl2 = ctypes.c_double(-1.0)
        assert L.gclaw_step_host(ctypes.byref(s), ptr(q), ptr(ref), dt, ctypes.c_void_p(base),
                                 nb, ctypes.byref(cfl2), stream) == 0
        assert np.array_equal(out, ref) and cfl.value == cfl2.value
