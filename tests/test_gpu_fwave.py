"""Shallow water over bathymetry in f-wave form (aux = (b,) per cell) on the
GPU against the oracle.

The -fmad=false build must reproduce the oracle bit for bit with every
boundary mix (q and aux), limiter, order and transverse option, on interior
and on ghost-filled (gclaw_step2) input; a lake at rest on dyadic depths
stays bit for bit at rest; the product build stays within 1e-13 per step,
FP32-bulk within 2e-6; a wave crossing a submerged ridge through the
PyClaw front end (solver.fwave = True) stays within 1e-12 of the oracle's
evolve at every frame."""
import ctypes

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, pyclaw, riemann
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import PD, random_bathymetry, random_state, rel_l1

pytestmark = pytest.mark.gpu
FW = _lib.RP_SHALLOW_BATHYMETRY_FWAVE_2D


def fw_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, order=2, tw=2, lim=4, precision=0,
            strict=False, pd=None):
    s = make_solver_struct(FW, q.shape[1], q.shape[2], dx, dy, bcl, bcu, [lim] * 3, order, tw,
                           precision, pd or PD[FW], abl, abu)
    dev = DeviceProblem(s, strict=strict, aux=aux)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


SIZES = [(2, 2), (3, 70), (37, 29), (96, 40), (70, 3)]
BCS = [((1, 1), (1, 1)), ((2, 2), (2, 2)), ((3, 3), (3, 3)), ((3, 1), (1, 3))]


@pytest.mark.parametrize("mx,my", SIZES)
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_ridge_strict_bitwise(cuda, oracle, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx * 37 + my)
    q = random_state(FW, mx, my, rng)
    aux = random_bathymetry(mx, my, rng)
    dx, dy = 1.0 / mx, 1.2 / my
    dt = 0.02 * min(dx, dy)
    lim = [1, 2, 3, 4][(mx + my) % 4]
    abl, abu = list(bcl), list(bcu)
    qo, cflo, rc = oracle.step_aux(FW, PD[FW], q, aux, dx, dy, dt, bcl, bcu, abl, abu, 2, 2,
                                   [lim] * 4)
    assert rc == 0
    qs, c = fw_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, lim=lim, strict=True)
    assert c.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    qp, cp = fw_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, lim=lim)
    assert rel_l1(qp, qo) <= 1e-13 and abs(cp.cfl - cflo) <= 1e-14 * cflo
    q32, c32 = fw_step(q, aux, dx, dy, dt, bcl, bcu, abl, abu, lim=lim, precision=1)
    assert rel_l1(q32, qo) <= 2e-6 and abs(c32.cfl - cflo) <= 1e-5 * cflo


@pytest.mark.parametrize("order,tw,lim", [(2, 2, 4), (2, 1, 2), (2, 0, 3), (1, 2, 0), (1, 0, 1),
                                          (2, 2, 0)])
def test_method_options_strict_bitwise(cuda, oracle, order, tw, lim):
    mx, my = 45, 33
    rng = np.random.default_rng(order * 7 + tw + lim)
    q = random_state(FW, mx, my, rng)
    aux = random_bathymetry(mx, my, rng)
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.01 / max(mx, my)
    bc = ([3, 1], [1, 3])
    qo, cflo, _ = oracle.step_aux(FW, PD[FW], q, aux, dx, dy, dt, *bc, [3, 1], [1, 3], order, tw,
                                  [lim] * 4)
    qs, c = fw_step(q, aux, dx, dy, dt, *bc, [3, 1], [1, 3], order, tw, lim, strict=True)
    assert np.array_equal(qs, qo)
    assert c.cfl == cflo


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("precision", [0, 1])
def test_lake_at_rest_exact(cuda, strict, precision):
    """Dyadic depths and bottoms with g = 1: every f-wave is exactly zero, in
    FP64 and in FP32, so the state does not change by a bit."""
    mx, my = 77, 53
    rng = np.random.default_rng(12)
    b = -(rng.integers(0, 8, size=(mx, my)) / 8.0)
    q = np.zeros((3, mx, my), order="F")
    q[0] = 2.0 - b
    aux = np.asfortranarray(b[None])
    qs, c = fw_step(q, aux, 0.1, 0.1, 0.01, [3, 3], [3, 3], [1, 1], [1, 1], precision=precision,
                    strict=strict, pd=[1.0])
    assert c.status == 0
    assert np.array_equal(qs, q)


def test_dry_cell_is_nonphysical(cuda):
    mx, my = 20, 20
    q = random_state(FW, mx, my, np.random.default_rng(1))
    q[0, 7, 9] = 0.0
    aux = np.zeros((1, mx, my), order="F")
    qs, c = fw_step(q, aux, 0.05, 0.05, 0.001, [1, 1], [1, 1], [1, 1], [1, 1])
    assert c.status == _lib.NONPHYSICAL


def test_step2_ghosted_input(cuda, oracle):
    mx, my = 41, 29
    rng = np.random.default_rng(8)
    q = random_state(FW, mx, my, rng)
    aux = random_bathymetry(mx, my, rng)
    bcl, bcu = [3, 2], [1, 2]
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    abc = oracle.fill_aux_ghosts(aux, bcl, bcu)
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.01 / max(mx, my)
    qo, cflo, rc = oracle.step_aux(FW, PD[FW], q, aux, dx, dy, dt, bcl, bcu, bcl, bcu)
    L = _lib.lib(strict=True)
    d_aux = torch.from_numpy(np.ascontiguousarray(abc.T)).cuda()
    s = make_solver_struct(FW, mx, my, dx, dy, bcl, bcu, [4] * 3, 2, 2, 0, PD[FW], bcl, bcu)
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


def test_split_refuses_fwave_solver(cuda):
    mx, my = 16, 16
    aux = random_bathymetry(mx, my, np.random.default_rng(0))
    s = make_solver_struct(FW, mx, my, 0.1, 0.1, [1, 1], [1, 1], [4] * 3, 2, 2, 0, PD[FW])
    with pytest.raises(_lib.GclawError):
        DeviceProblem(s, aux=aux, split=True).step(0.01)


def ridge_claw(mx=128, my=96, tfinal=0.3, nout=3):
    """A hump of water running over a submerged ridge between walls."""
    x = pyclaw.Dimension(-1.0, 1.0, mx, name="x")
    y = pyclaw.Dimension(-1.0, 1.0, my, name="y")
    domain = pyclaw.Domain([x, y])
    state = pyclaw.State(domain, 3, 1)
    state.problem_data["grav"] = 9.81
    X, Y = state.grid.p_centers
    state.aux[0] = -1.0 + 0.6 * np.exp(-30.0 * (X - 0.2 - 0.3 * Y) ** 2)
    state.q[0] = -state.aux[0] + 0.2 * np.exp(-40.0 * ((X + 0.5) ** 2 + Y ** 2))
    state.q[1] = 0.0
    state.q[2] = 0.0
    solver = pyclaw.ClawSolver2D(riemann.shallow_bathymetry_fwave_2D)
    solver.fwave = True
    solver.dimensional_split = False
    solver.transverse_waves = 2
    solver.limiters = pyclaw.limiters.tvd.MC
    solver.bc_lower = [pyclaw.BC.wall, pyclaw.BC.wall]
    solver.bc_upper = [pyclaw.BC.wall, pyclaw.BC.wall]
    solver.aux_bc_lower = [pyclaw.BC.wall, pyclaw.BC.wall]
    solver.aux_bc_upper = [pyclaw.BC.wall, pyclaw.BC.wall]
    solver.dt_initial = 0.002
    claw = pyclaw.Controller()
    claw.solution = pyclaw.Solution(state, domain)
    claw.solver = solver
    claw.tfinal, claw.num_output_times = tfinal, nout
    return claw


def test_ridge_problem_through_pyclaw_front_end(cuda, oracle):
    claw = ridge_claw()
    q0 = claw.solution.state.q.copy()
    aux = claw.solution.state.aux.copy()
    dx, dy = claw.solution.state.grid.delta
    claw.run()
    assert len(claw.frames) == 4

    def step(q, dt):
        qn, cfl, rc = oracle.step_aux(FW, [9.81], q, aux, dx, dy, dt, [3, 3], [3, 3], [3, 3],
                                      [3, 3], 2, 2, [4] * 3, nthreads=8)
        assert rc == 0
        return qn, cfl

    q, t, dt = q0, 0.0, 0.002
    for k in range(1, 4):
        q, t, dt, _ = oracle.evolve(step, q, t, 0.1 * k, dt, cfl_desired=0.9, cfl_max=1.0)
        assert rel_l1(claw.frames[k].q, q) <= 1e-12, k
    # mass is conserved between walls; the hump moved
    assert abs(claw.frames[-1].q[0].sum() - q0[0].sum()) <= 1e-12 * q0[0].sum()
    assert np.abs(claw.frames[-1].q[1]).max() > 1e-3


def test_front_end_checks_fwave_flag(cuda):
    claw = ridge_claw(16, 16, 0.01, 1)
    claw.solver.fwave = False
    with pytest.raises(ValueError):
        claw.run()
