"""The 3D steps (gclaw3_step / gclaw3_advance and their split forms,
acoustics_3D and euler_3D) on the GPU against the oracle's restatement of
classic3.

The -fmad=false build must reproduce the oracle bit for bit for every
transverse option (0, 10, 11, 20, 22), order, limiter and boundary mix,
including grids of 2 cells in a direction; the product build stays within
1e-13 per step and FP32-bulk within 2e-6; device-controlled time stepping
follows the oracle's evolve_to_time within 1e-12 (FP64) and 1e-6 (FP32);
unknown transverse options and precisions are refused.  The dimensionally
split step (ClawSolver3D's default) is held to the same bars against the
oracle's split sweeps."""
import ctypes
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib
from clawpack_gb300.device import DeviceProblem3, make_solver3_struct
from tests.helpers import rel_l1

pytestmark = pytest.mark.gpu
PD3 = [1.0, 4.0, 2.0, 2.0]


def gpu_step3(q, d, dt, bcl, bcu, order=2, tw=22, lim=4, strict=False, precision=0):
    m, mx, my, mz = q.shape
    s = make_solver3_struct(1, mx, my, mz, *d, bcl, bcu, [lim] * 2, order, tw, precision, PD3)
    dev = DeviceProblem3(s, strict=strict)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


SIZES = [(2, 2, 2), (5, 4, 3), (17, 9, 12), (24, 20, 6)]
BCS = [([1, 1, 1], [1, 1, 1]), ([2, 2, 2], [2, 2, 2]), ([3, 3, 3], [3, 3, 3]),
       ([3, 1, 2], [1, 3, 2])]


@pytest.mark.parametrize("shape", SIZES)
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_strict_bitwise(cuda, oracle, shape, bcl, bcu):
    rng = np.random.default_rng(sum(shape) + bcl[0])
    q = np.asfortranarray(rng.normal(size=(4,) + shape))
    d = (1.0 / shape[0], 1.1 / shape[1], 0.9 / shape[2])
    dt = 0.1 * min(d) / 2.0
    lim = [1, 2, 3, 4][sum(shape) % 4]
    qo, cflo = oracle.step3(1, PD3, q, *d, dt, bcl, bcu, 2, 22, [lim] * 2)
    qs, c = gpu_step3(q, d, dt, bcl, bcu, lim=lim, strict=True)
    assert c.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    qp, cp = gpu_step3(q, d, dt, bcl, bcu, lim=lim)
    assert rel_l1(qp, qo) <= 1e-13 and abs(cp.cfl - cflo) <= 1e-14 * cflo
    q32, c32 = gpu_step3(q, d, dt, bcl, bcu, lim=lim, precision=1)
    assert rel_l1(q32, qo) <= 2e-6 and abs(c32.cfl - cflo) <= 1e-6 * cflo


@pytest.mark.parametrize("order,tw,lim", [(2, 22, 4), (2, 20, 2), (2, 11, 3), (1, 10, 0),
                                          (2, 0, 1), (1, 0, 0), (2, 22, 0)])
def test_options_strict_bitwise(cuda, oracle, order, tw, lim):
    rng = np.random.default_rng(order * 100 + tw + lim)
    shape = (13, 11, 9)
    q = np.asfortranarray(rng.normal(size=(4,) + shape))
    d = (0.1, 0.12, 0.09)
    dt = 0.02
    bcl, bcu = [3, 1, 2], [1, 3, 2]
    qo, cflo = oracle.step3(1, PD3, q, *d, dt, bcl, bcu, order, tw, [lim] * 2)
    qs, c = gpu_step3(q, d, dt, bcl, bcu, order, tw, lim, strict=True)
    assert np.array_equal(qs, qo)
    assert c.cfl == cflo


def test_device_controlled_evolve(cuda, oracle):
    """A radial pressure pulse between walls: 0.3 time units under the
    evolve_to_time rules on the device against the oracle's loop."""
    mx, my, mz = 24, 20, 16
    x = (np.arange(mx) + 0.5) / mx - 0.5
    y = (np.arange(my) + 0.5) / my - 0.5
    z = (np.arange(mz) + 0.5) / mz - 0.5
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    q = np.zeros((4, mx, my, mz), order="F")
    q[0] = np.exp(-40.0 * (X ** 2 + Y ** 2 + Z ** 2))
    d = (1.0 / mx, 1.0 / my, 1.0 / mz)
    bc = [3, 3, 3]
    s = make_solver3_struct(1, mx, my, mz, *d, bc, bc, [4, 4], 2, 22, 0, PD3)
    dev = DeviceProblem3(s)
    dev.upload(q)
    c = dev.evolve(0.0, 0.002, 0.3, cfl_max=1.0, cfl_desired=0.9)
    assert c.status == 0

    def step(qq, dt):
        return oracle.step3(1, PD3, qq, *d, dt, bc, bc, 2, 22, [4, 4], nthreads=8)

    qo, t, dt, info = oracle.evolve(step, q, 0.0, 0.3, 0.002, cfl_desired=0.9, cfl_max=1.0)
    assert c.numsteps == info["numsteps"]
    assert rel_l1(dev.download(c.parity), qo) <= 1e-12
    # acoustic energy stays bounded and the pulse spread out
    assert np.abs(dev.download(c.parity)[0]).max() < 0.5


def test_refusals(cuda):
    L = _lib.lib()
    s = make_solver3_struct(1, 8, 8, 8, 0.1, 0.1, 0.1, [1] * 3, [1] * 3, [4, 4], 2, 21, 0, PD3)
    assert L.gclaw3_check(ctypes.byref(s)) == _lib.ERR_UNSUPPORTED
    s.transverse_waves = 22
    s.precision = 2
    assert L.gclaw3_check(ctypes.byref(s)) == _lib.ERR_UNSUPPORTED
    s.precision = 1  # FP32-bulk: half the workspace
    assert L.gclaw3_check(ctypes.byref(s)) == 0
    b32 = L.gclaw3_workspace_bytes(ctypes.byref(s))
    s.precision = 0
    assert L.gclaw3_check(ctypes.byref(s)) == 0
    assert L.gclaw3_workspace_bytes(ctypes.byref(s)) == 2 * b32
    s.mz = 1
    assert L.gclaw3_check(ctypes.byref(s)) == _lib.ERR_ARG


def test_controller_run_through_clawsolver3d(cuda, oracle):
    from clawpack_gb300 import pyclaw, riemann

    dims = [pyclaw.Dimension(-1.0, 1.0, n, name=c) for n, c in ((20, "x"), (18, "y"), (16, "z"))]
    domain = pyclaw.Domain(dims)
    state = pyclaw.State(domain, 4)
    state.problem_data.update(rho=1.0, bulk=4.0)
    X, Y, Z = state.grid.p_centers
    state.q[0] = np.exp(-20.0 * ((X - 0.2) ** 2 + Y ** 2 + (Z + 0.1) ** 2))
    solver = pyclaw.ClawSolver3D(riemann.acoustics_3D)
    solver.dimensional_split = False
    solver.limiters = pyclaw.limiters.tvd.MC
    solver.bc_lower = [pyclaw.BC.extrap, pyclaw.BC.wall, pyclaw.BC.periodic]
    solver.bc_upper = [pyclaw.BC.extrap, pyclaw.BC.wall, pyclaw.BC.periodic]
    solver.dt_initial = 0.01
    claw = pyclaw.Controller()
    claw.solution = pyclaw.Solution(state, domain)
    claw.solver = solver
    claw.tfinal, claw.num_output_times = 0.3, 3
    q0 = state.q.copy()
    claw.run()
    d = tuple(state.grid.delta)
    bcl, bcu = [1, 3, 2], [1, 3, 2]

    def step(qq, dt):
        return oracle.step3(1, PD3, qq, *d, dt, bcl, bcu, 2, 22, [4, 4], nthreads=8)

    q, t, dt = q0, 0.0, 0.01
    for k in range(1, 4):
        q, t, dt, _ = oracle.evolve(step, q, t, 0.1 * k, dt, cfl_desired=0.9, cfl_max=1.0)
        assert rel_l1(claw.frames[k].q, q) <= 1e-12, k


def test_fp32_bulk_evolve(cuda, oracle):
    mx, my, mz = 24, 20, 16
    x = (np.arange(mx) + 0.5) / mx - 0.5
    y = (np.arange(my) + 0.5) / my - 0.5
    z = (np.arange(mz) + 0.5) / mz - 0.5
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    q = np.zeros((4, mx, my, mz), order="F")
    q[0] = np.exp(-40.0 * (X ** 2 + Y ** 2 + Z ** 2))
    d = (1.0 / mx, 1.0 / my, 1.0 / mz)
    bc = [3, 3, 3]
    res = {}
    for prec in (0, 1):
        s = make_solver3_struct(1, mx, my, mz, *d, bc, bc, [4, 4], 2, 22, prec, PD3)
        dev = DeviceProblem3(s)
        dev.upload(q)
        c = dev.evolve(0.0, 0.002, 0.3, cfl_max=1.0, cfl_desired=0.9)
        assert c.status == 0
        res[prec] = (dev.download(c.parity), c)
    assert res[0][1].numsteps == res[1][1].numsteps
    assert rel_l1(res[1][0], res[0][0]) <= 1e-6


# ---------------------------------------------------------------------------
# euler_3D
# ---------------------------------------------------------------------------
def euler3(shape, rng, gamma=1.4):
    rho = 0.5 + rng.random(shape)
    u = 0.5 * rng.normal(size=(3,) + shape)
    p = 0.5 + rng.random(shape)
    q = np.empty((5,) + shape, order="F")
    q[0] = rho
    q[1:4] = rho * u
    q[4] = p / (gamma - 1.0) + 0.5 * rho * (u ** 2).sum(axis=0)
    return q


def gpu_euler3(q, d, dt, bcl, bcu, order=2, tw=22, lim=4, strict=False, precision=0):
    m, mx, my, mz = q.shape
    s = make_solver3_struct(2, mx, my, mz, *d, bcl, bcu, [lim] * 3, order, tw, precision, [1.4])
    dev = DeviceProblem3(s, strict=strict)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


@pytest.mark.parametrize("shape", [(2, 2, 2), (5, 4, 3), (17, 9, 12)])
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_euler_strict_bitwise(cuda, oracle, shape, bcl, bcu):
    rng = np.random.default_rng(7 * sum(shape) + bcl[0])
    q = euler3(shape, rng)
    d = (1.0 / shape[0], 1.1 / shape[1], 0.9 / shape[2])
    dt = 0.05 * min(d)
    lim = [1, 2, 3, 4][sum(shape) % 4]
    qo, cflo = oracle.step3(2, [1.4], q, *d, dt, bcl, bcu, 2, 22, [lim] * 3)
    qs, c = gpu_euler3(q, d, dt, bcl, bcu, lim=lim, strict=True)
    assert c.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    qp, cp = gpu_euler3(q, d, dt, bcl, bcu, lim=lim)
    assert rel_l1(qp, qo) <= 1e-13 and abs(cp.cfl - cflo) <= 1e-14 * cflo
    q32, c32 = gpu_euler3(q, d, dt, bcl, bcu, lim=lim, precision=1)
    assert rel_l1(q32, qo) <= 2e-6 and abs(c32.cfl - cflo) <= 1e-6 * cflo


@pytest.mark.parametrize("order,tw,lim", [(2, 20, 2), (2, 11, 3), (1, 10, 0), (2, 0, 1)])
def test_euler_options_strict_bitwise(cuda, oracle, order, tw, lim):
    rng = np.random.default_rng(order * 100 + tw + lim + 1)
    q = euler3((13, 11, 9), rng)
    d = (0.1, 0.12, 0.09)
    dt = 0.004
    bcl, bcu = [3, 1, 2], [1, 3, 2]
    qo, cflo = oracle.step3(2, [1.4], q, *d, dt, bcl, bcu, order, tw, [lim] * 3)
    qs, c = gpu_euler3(q, d, dt, bcl, bcu, order, tw, lim, strict=True)
    assert np.array_equal(qs, qo)
    assert c.cfl == cflo


def test_euler_nonphysical_state(cuda):
    rng = np.random.default_rng(3)
    q = euler3((8, 8, 8), rng)
    q[4, 3, 4, 5] = 0.01 * q[4, 3, 4, 5] - 5.0  # negative pressure
    qs, c = gpu_euler3(q, (0.1, 0.1, 0.1), 0.001, [1] * 3, [1] * 3)
    assert c.status == _lib.NONPHYSICAL


def test_euler_clawsolver3d_run(cuda, oracle):
    """A spherical over-pressure between walls through ClawSolver3D."""
    from clawpack_gb300 import pyclaw, riemann

    dims = [pyclaw.Dimension(-1.0, 1.0, n, name=c) for n, c in ((18, "x"), (16, "y"), (14, "z"))]
    domain = pyclaw.Domain(dims)
    state = pyclaw.State(domain, 5)
    state.problem_data["gamma"] = 1.4
    X, Y, Z = state.grid.p_centers
    p = 1.0 + 2.0 * (X ** 2 + Y ** 2 + Z ** 2 < 0.25)
    state.q[0] = 1.0
    state.q[4] = p / 0.4
    solver = pyclaw.ClawSolver3D(riemann.euler_3D)
    solver.dimensional_split = False
    solver.limiters = pyclaw.limiters.tvd.MC
    solver.bc_lower = [pyclaw.BC.wall] * 3
    solver.bc_upper = [pyclaw.BC.wall] * 3
    solver.dt_initial = 0.005
    claw = pyclaw.Controller()
    claw.solution = pyclaw.Solution(state, domain)
    claw.solver = solver
    claw.tfinal, claw.num_output_times = 0.2, 2
    q0 = state.q.copy()
    claw.run()
    d = tuple(state.grid.delta)

    def step(qq, dt):
        return oracle.step3(2, [1.4], qq, *d, dt, [3] * 3, [3] * 3, 2, 22, [4] * 3, nthreads=8)

    q, t, dt = q0, 0.0, 0.005
    for k in range(1, 3):
        q, t, dt, _ = oracle.evolve(step, q, t, 0.1 * k, dt, cfl_desired=0.9, cfl_max=1.0)
        assert rel_l1(claw.frames[k].q, q) <= 1e-12, k
    # mass and energy are conserved between walls
    for comp in (0, 4):
        assert abs(claw.frames[-1].q[comp].sum() - q0[comp].sum()) <= 1e-12 * q0[comp].sum()


# ---------------------------------------------------------------------------
# dimensionally split steps (gclaw3_step_split / gclaw3_advance_split)
# ---------------------------------------------------------------------------
def gpu_split3(rp, pd, q, d, dt, bcl, bcu, order=2, lim=4, strict=False, precision=0):
    m, mx, my, mz = q.shape
    s = make_solver3_struct(rp, mx, my, mz, *d, bcl, bcu, [lim] * 3, order, 22, precision, pd)
    dev = DeviceProblem3(s, strict=strict, split=True)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


@pytest.mark.parametrize("shape", [(2, 2, 2), (5, 4, 3), (17, 9, 12)])
@pytest.mark.parametrize("bcl,bcu", BCS)
@pytest.mark.parametrize("rp", [1, 2])
def test_split_strict_bitwise(cuda, oracle, rp, shape, bcl, bcu):
    rng = np.random.default_rng(11 * sum(shape) + bcl[0] + rp)
    if rp == 1:
        q, pd = np.asfortranarray(rng.normal(size=(4,) + shape)), PD3
    else:
        q, pd = euler3(shape, rng), [1.4]
    d = (1.0 / shape[0], 1.1 / shape[1], 0.9 / shape[2])
    dt = (0.05 if rp == 1 else 0.04) * min(d)
    lim = [1, 2, 3, 4][sum(shape) % 4]
    qo, cflo = oracle.step3_split(rp, pd, q, *d, dt, bcl, bcu, 2, [lim] * 3)
    qs, c = gpu_split3(rp, pd, q, d, dt, bcl, bcu, lim=lim, strict=True)
    assert c.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    qp, cp = gpu_split3(rp, pd, q, d, dt, bcl, bcu, lim=lim)
    assert rel_l1(qp, qo) <= 1e-13 and abs(cp.cfl - cflo) <= 1e-14 * cflo
    q32, c32 = gpu_split3(rp, pd, q, d, dt, bcl, bcu, lim=lim, precision=1)
    assert rel_l1(q32, qo) <= 2e-6 and abs(c32.cfl - cflo) <= 1e-6 * cflo


@pytest.mark.parametrize("shape", [(130, 6, 5), (61, 34, 4), (5, 70, 3), (4, 3, 67)])
@pytest.mark.parametrize("rp", [1, 2])
def test_split_long_pencils(cuda, oracle, rp, shape):
    """Pencils longer than a chunk (16 cells in FP32, 32 in FP64) and than
    the x-sweep's warp windows (28 cells, four per warp)."""
    rng = np.random.default_rng(sum(shape) + rp)
    if rp == 1:
        q, pd = np.asfortranarray(rng.normal(size=(4,) + shape)), PD3
    else:
        q, pd = euler3(shape, rng), [1.4]
    d = (1.0 / shape[0], 1.0 / shape[1], 1.0 / shape[2])
    dt = 0.04 * min(d)
    bcl, bcu = [3, 2, 1], [1, 2, 3]
    qo, cflo = oracle.step3_split(rp, pd, q, *d, dt, bcl, bcu, 2, [4] * 3, nthreads=4)
    qs, c = gpu_split3(rp, pd, q, d, dt, bcl, bcu, strict=True)
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    q32, c32 = gpu_split3(rp, pd, q, d, dt, bcl, bcu, precision=1)
    assert rel_l1(q32, qo) <= 2e-6 and abs(c32.cfl - cflo) <= 1e-6 * cflo


@pytest.mark.parametrize("order,lim", [(1, 0), (2, 1), (2, 0)])
def test_split_options_strict_bitwise(cuda, oracle, order, lim):
    rng = np.random.default_rng(order * 10 + lim)
    q = np.asfortranarray(rng.normal(size=(4, 13, 11, 9)))
    d = (0.1, 0.12, 0.09)
    bcl, bcu = [3, 1, 2], [1, 3, 2]
    qo, cflo = oracle.step3_split(1, PD3, q, *d, 0.02, bcl, bcu, order, [lim] * 3)
    qs, c = gpu_split3(1, PD3, q, d, 0.02, bcl, bcu, order, lim, strict=True)
    assert np.array_equal(qs, qo)
    assert c.cfl == cflo


def test_split_refusals(cuda):
    L = _lib.lib()
    s = make_solver3_struct(1, 8, 8, 8, 0.1, 0.1, 0.1, [1] * 3, [1] * 3, [4, 4], 2, 22, 0, PD3)
    dev = DeviceProblem3(s, split=True)
    p = [ctypes.c_void_p(t.data_ptr()) for t in (dev.q[0], dev.q[1], dev.qtmp)]
    ws, ctrl = ctypes.c_void_p(dev.ws.data_ptr()), ctypes.c_void_p(dev.ctrl.data_ptr())
    sp = ctypes.byref(s)
    assert L.gclaw3_step_split(sp, p[0], p[1], p[0], 0.01, ws, ctrl, None) == _lib.ERR_ARG
    assert L.gclaw3_step_split(sp, p[0], p[1], None, 0.01, ws, ctrl, None) == _lib.ERR_ARG
    assert L.gclaw3_step_split(sp, p[0], p[1], p[2], 0.0, ws, ctrl, None) == _lib.ERR_ARG
    assert L.gclaw3_advance_split(sp, p[0], p[1], p[1], ws, ctrl, 1, None) == _lib.ERR_ARG
    assert L.gclaw3_advance_split(sp, p[0], p[1], p[2], ws, ctrl, -1, None) == _lib.ERR_ARG
    # state arrays off a 16-byte boundary are refused before any launch
    off = ctypes.c_void_p(dev.q[1].data_ptr() + 8)
    assert L.gclaw3_step_split(sp, p[0], off, p[2], 0.01, ws, ctrl, None) == _lib.ERR_ARG
    assert L.gclaw3_advance_split(sp, off, p[0], p[2], ws, ctrl, 1, None) == _lib.ERR_ARG
    big = torch.zeros(2 * dev.q[0].numel() + 2, dtype=torch.float64, device="cuda")
    b0, b1 = (ctypes.c_void_p(big.data_ptr() + 8), ctypes.c_void_p(big.data_ptr() + 8 * (dev.q[0].numel() + 2)))
    s.transverse_waves = 0
    wsu = torch.empty(L.gclaw3_workspace_bytes(sp), dtype=torch.uint8, device="cuda")
    assert L.gclaw3_step(sp, b0, b1, 0.01, ctypes.c_void_p(wsu.data_ptr()), ctrl, None) == _lib.ERR_ARG
    assert L.gclaw3_advance(sp, b0, b1, ctypes.c_void_p(wsu.data_ptr()), ctrl, 1, None) == _lib.ERR_ARG
    # split steps need no workspace
    dev.upload(np.zeros((4, 8, 8, 8), order="F"))
    assert L.gclaw3_step_split(sp, p[0], p[1], p[2], 0.01, None, ctrl, None) == 0
    torch.cuda.synchronize()


def test_split_clawsolver3d_run(cuda, oracle):
    """ClawSolver3D's default (dimensional_split = True): an acoustic pulse
    between mixed boundaries through the Controller against the oracle's
    split steps under evolve_to_time."""
    from clawpack_gb300 import pyclaw, riemann

    dims = [pyclaw.Dimension(-1.0, 1.0, n, name=c) for n, c in ((20, "x"), (18, "y"), (16, "z"))]
    domain = pyclaw.Domain(dims)
    state = pyclaw.State(domain, 4)
    state.problem_data.update(rho=1.0, bulk=4.0)
    X, Y, Z = state.grid.p_centers
    state.q[0] = np.exp(-20.0 * ((X - 0.2) ** 2 + Y ** 2 + (Z + 0.1) ** 2))
    solver = pyclaw.ClawSolver3D(riemann.acoustics_3D)
    assert solver.dimensional_split
    solver.limiters = pyclaw.limiters.tvd.MC
    solver.bc_lower = [pyclaw.BC.extrap, pyclaw.BC.wall, pyclaw.BC.periodic]
    solver.bc_upper = [pyclaw.BC.extrap, pyclaw.BC.wall, pyclaw.BC.periodic]
    solver.dt_initial = 0.01
    claw = pyclaw.Controller()
    claw.solution = pyclaw.Solution(state, domain)
    claw.solver = solver
    claw.tfinal, claw.num_output_times = 0.3, 3
    q0 = state.q.copy()
    claw.run()
    d = tuple(state.grid.delta)
    bcl, bcu = [1, 3, 2], [1, 3, 2]

    def step(qq, dt):
        return oracle.step3_split(1, PD3, qq, *d, dt, bcl, bcu, 2, [4, 4], nthreads=8)

    q, t, dt = q0, 0.0, 0.01
    for k in range(1, 4):
        q, t, dt, _ = oracle.evolve(step, q, t, 0.1 * k, dt, cfl_desired=0.9, cfl_max=1.0)
        assert rel_l1(claw.frames[k].q, q) <= 1e-12, k


@pytest.mark.parametrize("rp", [1, 2])
@pytest.mark.parametrize("precision", [0, 1])
def test_split_pencil_kernels_agree(cuda, rp, precision):
    """Marching threads (gclaw3_split_kernel(1), the default) and warp
    windows (2) along y and z give bit-identical split steps in the strict
    build, on pencils longer than four windows."""
    shape = (9, 130, 117)
    rng = np.random.default_rng(rp + 3 * precision)
    if rp == 1:
        q, pd = np.asfortranarray(rng.normal(size=(4,) + shape)), PD3
    else:
        q, pd = euler3(shape, rng), [1.4]
    d = (0.1, 1.0 / 130, 1.0 / 117)
    dt = 0.04 * min(d)
    L = _lib.lib(True)
    res = {}
    for fam in (1, 2, 0):
        prev = L.gclaw3_split_kernel(fam)
        try:
            res[fam] = gpu_split3(rp, pd, q, d, dt, [3, 1, 2], [1, 3, 2], strict=True,
                                  precision=precision)
        finally:
            L.gclaw3_split_kernel(prev)
    for fam in (1, 2):
        assert np.array_equal(res[fam][0], res[0][0]), fam
        assert res[fam][1].cfl == res[0][1].cfl and res[fam][1].status == res[0][1].status == 0


@pytest.mark.parametrize("shape", [(40, 13, 20), (7, 33, 9), (2, 2, 2), (31, 7, 17)])
@pytest.mark.parametrize("rp,tw", [(1, 22), (1, 11), (1, 20), (1, 10), (2, 22), (2, 11), (2, 20)])
def test_slab_and_staged_agree(cuda, rp, tw, shape):
    """FP32-bulk sweeps with transverse terms: the fused slab kernel (the
    default) and the staged kernels (gclaw3_unsplit_kernel(1)) give
    bit-identical steps in the strict build, on grids of several tiles and
    chunks and on ragged ones, for every transverse option."""
    rng = np.random.default_rng(sum(shape) + tw + rp)
    if rp == 1:
        q, pd = np.asfortranarray(rng.normal(size=(4,) + shape)), PD3
    else:
        q, pd = euler3(shape, rng), [1.4]
    d = (1.0 / shape[0], 1.1 / shape[1], 0.9 / shape[2])
    dt = 0.04 * min(d)
    L = _lib.lib(True)
    res = {}
    for fam in (1, 0):
        prev = L.gclaw3_unsplit_kernel(fam)
        try:
            m, mx, my, mz = q.shape
            s = make_solver3_struct(rp, mx, my, mz, *d, [3, 1, 2], [1, 3, 2], [4] * 3, 2, tw, 1,
                                    pd)
            dev = DeviceProblem3(s, strict=True)
            dev.upload(q)
            dev.step(dt, src=0)
            res[fam] = (dev.download(1), dev.read_ctrl())
        finally:
            L.gclaw3_unsplit_kernel(prev)
    assert np.array_equal(res[0][0], res[1][0]), np.abs(res[0][0] - res[1][0]).max()
    assert res[0][1].cfl == res[1][1].cfl and res[0][1].status == res[1][1].status == 0
