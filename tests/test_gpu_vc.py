"""Variable-coefficient acoustics (aux = (rho, c) per cell) on the GPU
against the oracle.

The -fmad=false build must reproduce the oracle bit for bit on layered
random media with every boundary mix (q and aux), limiter, order and
transverse option, on interior and on ghost-filled (gclaw_step2) input; a
constant medium must give constant-coefficient acoustics bit for bit; the
product build stays within 1e-13 per step, FP32-bulk within 2e-6; a
Controller run through the PyClaw front end stays within 1e-12 of the
oracle's evolve at every frame."""
import ctypes
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, pyclaw, riemann
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import PD, random_medium, random_state, rel_l1

pytestmark = pytest.mark.gpu
VC = _lib.RP_VC_ACOUSTICS_2D


def vc_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, order=2, tw=2, lim=4, precision=0,
            strict=False):
    s = make_solver_struct(VC, q.shape[1], q.shape[2], dx, dy, bcl, bcu, [lim] * 2, order, tw,
                           precision, [], abl, abu)
    dev = DeviceProblem(s, strict=strict, aux=aux)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


SIZES = [(2, 2), (3, 70), (37, 29), (96, 40)]
BCS = [((1, 1), (1, 1)), ((2, 2), (2, 2)), ((3, 3), (3, 3)), ((3, 1), (1, 3))]


@pytest.mark.parametrize("mx,my", SIZES)
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_layered_medium_strict_bitwise(cuda, oracle, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx * 31 + my)
    q = random_state(1, mx, my, rng)
    aux = random_medium(mx, my, rng)
    dx, dy = 1.0 / mx, 1.2 / my
    dt = 0.05 * min(dx, dy)
    lim = [1, 2, 3, 4][(mx + my) % 4]
    abl, abu = list(bcl), list(bcu)
    qo, cflo, rc = oracle.step_aux(VC, [], q, aux, dx, dy, dt, bcl, bcu, abl, abu, 2, 2,
                                   [lim] * 4)
    assert rc == 0
    qs, c = vc_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, lim=lim, strict=True)
    assert c.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    qp, cp = vc_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, lim=lim)
    assert rel_l1(qp, qo) <= 1e-13 and abs(cp.cfl - cflo) <= 1e-14 * cflo
    q32, c32 = vc_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, lim=lim, precision=1)
    assert rel_l1(q32, qo) <= 2e-6 and abs(c32.cfl - cflo) <= 1e-5 * cflo


@pytest.mark.parametrize("order,tw,lim", [(2, 2, 4), (2, 1, 2), (2, 0, 3), (1, 2, 0), (1, 0, 1)])
def test_method_options_strict_bitwise(cuda, oracle, order, tw, lim):
    mx, my = 45, 33
    rng = np.random.default_rng(order * 7 + tw + lim)
    q = random_state(1, mx, my, rng)
    aux = random_medium(mx, my, rng)
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.03 / max(mx, my)
    bc = ([3, 1], [1, 3])
    qo, cflo, _ = oracle.step_aux(VC, [], q, aux, dx, dy, dt, *bc, [1, 3], [3, 1], order, tw,
                                  [lim] * 4)
    qs, c = vc_step(q, aux, dx, dy, dt, *bc, [1, 3], [3, 1], order, tw, lim, strict=True)
    assert np.array_equal(qs, qo)
    assert c.cfl == cflo


def test_constant_medium_equals_acoustics(cuda):
    mx, my = 50, 37
    rng = np.random.default_rng(3)
    q = random_state(1, mx, my, rng)
    rho, bulk = 1.7, 5.3
    c = math.sqrt(bulk / rho)
    aux = np.empty((2, mx, my), order="F")
    aux[0], aux[1] = rho, c
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.02 / max(mx, my)
    qv, cv = vc_step(q, aux, dx, dy, dt, [3, 1], [1, 3], [3, 1], [1, 3], strict=True)
    s = make_solver_struct(1, mx, my, dx, dy, [3, 1], [1, 3], [4, 4], 2, 2, 0,
                           [rho, bulk, c, rho * c])
    dev = DeviceProblem(s, strict=True)
    dev.upload(q)
    dev.step(dt, src=0)
    assert np.array_equal(qv, dev.download(1))
    assert cv.cfl == dev.read_ctrl().cfl


def test_step2_ghosted_input(cuda, oracle):
    mx, my = 41, 29
    rng = np.random.default_rng(8)
    q = random_state(1, mx, my, rng)
    aux = random_medium(mx, my, rng)
    bcl, bcu = [3, 2], [1, 2]
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    abc = oracle.fill_aux_ghosts(aux, bcl, bcu)
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.02 / max(mx, my)
    qo, cflo, rc = oracle.step_aux(VC, [], q, aux, dx, dy, dt, bcl, bcu, bcl, bcu)
    L = _lib.lib(strict=True)
    d_aux = torch.from_numpy(np.ascontiguousarray(abc.T)).cuda()
    s = make_solver_struct(VC, mx, my, dx, dy, bcl, bcu, [4, 4], 2, 2, 0, [], bcl, bcu)
    s.aux = d_aux.data_ptr()
    d_in = torch.from_numpy(np.ascontiguousarray(qbc.T)).cuda()
    d_out = d_in.clone()
    ws = torch.zeros(_lib.CTRL_BYTES, dtype=torch.uint8, device="cuda")
    cfl = ctypes.c_double()
    rc = L.gclaw_step2(ctypes.byref(s), ctypes.c_void_p(d_in.data_ptr()),
                       ctypes.c_void_p(d_out.data_ptr()), dt, ctypes.c_void_p(ws.data_ptr()),
                       ctypes.byref(cfl), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    out = d_out.cpu().numpy().T
    assert np.array_equal(out[:, 2:-2, 2:-2], qo)
    assert cfl.value == cflo


def test_split_and_batched_refuse_aux_solvers(cuda):
    mx, my = 16, 16
    aux = random_medium(mx, my, np.random.default_rng(0))
    s = make_solver_struct(VC, mx, my, 0.1, 0.1, [1, 1], [1, 1], [4, 4], 2, 2, 0, [])
    dev = DeviceProblem(s, aux=aux)
    with pytest.raises(_lib.GclawError):
        DeviceProblem(s, aux=aux, split=True).step(0.01)
    assert dev.q[0].shape == (my, mx, 3)


def interface_claw(mx=120, my=100, tfinal=0.4, nout=4):
    """A plane pressure pulse crossing a tilted interface between two media."""
    x = pyclaw.Dimension(-1.0, 1.0, mx, name="x")
    y = pyclaw.Dimension(-1.0, 1.0, my, name="y")
    domain = pyclaw.Domain([x, y])
    state = pyclaw.State(domain, 3, 2)
    X, Y = state.grid.p_centers
    right = X + 0.3 * Y > 0.2
    state.aux[0] = np.where(right, 4.0, 1.0)  # density
    state.aux[1] = np.where(right, 0.5, 1.0)  # sound speed
    state.q[0] = np.exp(-100.0 * (X + 0.5) ** 2)
    state.q[1] = state.q[0] / (state.aux[0] * state.aux[1])  # right-going: u = p / Z
    solver = pyclaw.ClawSolver2D(riemann.vc_acoustics_2D)
    solver.dimensional_split = False
    solver.transverse_waves = 2
    solver.limiters = pyclaw.limiters.tvd.MC
    solver.bc_lower = [pyclaw.BC.extrap, pyclaw.BC.wall]
    solver.bc_upper = [pyclaw.BC.extrap, pyclaw.BC.wall]
    solver.aux_bc_lower = [pyclaw.BC.extrap, pyclaw.BC.wall]
    solver.aux_bc_upper = [pyclaw.BC.extrap, pyclaw.BC.wall]
    solver.dt_initial = 0.005
    claw = pyclaw.Controller()
    claw.solution = pyclaw.Solution(state, domain)
    claw.solver = solver
    claw.tfinal, claw.num_output_times = tfinal, nout
    return claw


def test_interface_problem_through_pyclaw_front_end(cuda, oracle):
    claw = interface_claw()
    q0 = claw.solution.state.q.copy()
    aux = claw.solution.state.aux.copy()
    dx, dy = claw.solution.state.grid.delta
    claw.run()
    assert len(claw.frames) == 5

    def step(q, dt):
        qn, cfl, rc = oracle.step_aux(VC, [], q, aux, dx, dy, dt, [1, 3], [1, 3], [1, 3], [1, 3],
                                      2, 2, [4, 4], nthreads=8)
        assert rc == 0
        return qn, cfl

    q, t, dt = q0, 0.0, 0.005
    for k in range(1, 5):
        q, t, dt, _ = oracle.evolve(step, q, t, 0.1 * k, dt, cfl_desired=0.9, cfl_max=1.0)
        assert rel_l1(claw.frames[k].q, q) <= 1e-12, k
    # the pulse reached the slower medium: part of it was reflected
    assert np.abs(claw.frames[-1].q[0]).max() > 0.1
