"""The capacity form of the step (a capacity kappa per cell, the last aux
field; classic2's mcapa) on the GPU against the oracle.

The -fmad=false build must reproduce the oracle bit for bit for every
solver (kappa alone for the solvers without aux, after the medium or the
bottom for the aux solvers), boundary mix, method option and ghost-filled
input; the product build stays within 1e-13 per step; device-controlled
time stepping through the PyClaw front end (state.index_capa) follows the
oracle's evolve within 1e-12; the entry points without a capacity form
refuse it."""
import ctypes
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, pyclaw, riemann
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import (PD, SHAPES, random_bathymetry, random_medium, random_state,
                           rel_l1)

pytestmark = pytest.mark.gpu
VC, FW = _lib.RP_VC_ACOUSTICS_2D, _lib.RP_SHALLOW_BATHYMETRY_FWAVE_2D
NUA = {1: 0, 2: 0, 3: 0, VC: 2, FW: 1}


def kappa(mx, my, rng):
    x = (np.arange(mx)[:, None] + 0.5) / mx
    y = (np.arange(my)[None, :] + 0.5) / my
    return 1.2 + 0.6 * np.sin(2 * math.pi * x) * np.cos(2 * math.pi * y) + \
        0.1 * rng.random((mx, my))


def problem(rp, mx, my, rng):
    q = random_state(rp, mx, my, rng)
    aux = np.empty((NUA[rp] + 1, mx, my), order="F")
    if rp == VC:
        aux[:2] = random_medium(mx, my, rng)
    elif rp == FW:
        aux[:1] = random_bathymetry(mx, my, rng)
    aux[-1] = kappa(mx, my, rng)
    return q, aux


def capa_step(rp, q, aux, dx, dy, dt, bcl, bcu, order=2, tw=2, lim=4, strict=False,
              precision=0):
    s = make_solver_struct(rp, q.shape[1], q.shape[2], dx, dy, bcl, bcu,
                           [lim] * SHAPES[rp][1], order, tw, precision, PD[rp], bcl, bcu,
                           capa=NUA[rp] + 1)
    dev = DeviceProblem(s, strict=strict, aux=aux)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


SIZES = [(2, 2), (3, 70), (37, 29), (96, 40)]
BCS = [((1, 1), (1, 1)), ((2, 2), (2, 2)), ((3, 3), (3, 3)), ((3, 1), (1, 3))]


@pytest.mark.parametrize("rp", [1, 2, 3, VC, FW])
@pytest.mark.parametrize("mx,my", SIZES)
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_capacity_strict_bitwise(cuda, oracle, rp, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx * 13 + my + 7 * rp)
    q, aux = problem(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.2 / my
    dt = 0.01 * min(dx, dy)
    lim = [1, 2, 3, 4][(mx + my) % 4]
    qo, cflo, rc = oracle.step_aux(rp, PD[rp], q, aux, dx, dy, dt, bcl, bcu, bcl, bcu, 2, 2,
                                   [lim] * 4, mcapa=NUA[rp] + 1)
    assert rc == 0
    qs, c = capa_step(rp, q, aux, dx, dy, dt, bcl, bcu, lim=lim, strict=True)
    assert c.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    qp, cp = capa_step(rp, q, aux, dx, dy, dt, bcl, bcu, lim=lim)
    assert rel_l1(qp, qo) <= 1e-13 and abs(cp.cfl - cflo) <= 1e-14 * cflo


@pytest.mark.parametrize("rp", [1, 2, 3, VC, FW])
@pytest.mark.parametrize("order,tw,lim", [(2, 1, 2), (2, 0, 3), (1, 2, 0), (1, 0, 1)])
def test_capacity_method_options(cuda, oracle, rp, order, tw, lim):
    mx, my = 45, 33
    rng = np.random.default_rng(order * 7 + tw + lim + rp)
    q, aux = problem(rp, mx, my, rng)
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.01 / max(mx, my)
    bcl, bcu = [3, 1], [1, 3]
    qo, cflo, _ = oracle.step_aux(rp, PD[rp], q, aux, dx, dy, dt, bcl, bcu, bcl, bcu, order, tw,
                                  [lim] * 4, mcapa=NUA[rp] + 1)
    qs, c = capa_step(rp, q, aux, dx, dy, dt, bcl, bcu, order, tw, lim, strict=True)
    assert np.array_equal(qs, qo)
    assert c.cfl == cflo


def test_capacity_step2_ghosted_input(cuda, oracle):
    rp, mx, my = 2, 41, 29
    rng = np.random.default_rng(8)
    q, aux = problem(rp, mx, my, rng)
    bcl, bcu = [3, 2], [1, 2]
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    abc = oracle.fill_aux_ghosts(aux, bcl, bcu)
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.01 / max(mx, my)
    qo, cflo, rc = oracle.step_aux(rp, PD[rp], q, aux, dx, dy, dt, bcl, bcu, bcl, bcu, mcapa=1)
    L = _lib.lib(strict=True)
    d_aux = torch.from_numpy(np.ascontiguousarray(abc.T)).cuda()
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [4] * 3, 2, 2, 0, PD[rp], bcl, bcu,
                           capa=1)
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


def test_capacity_refusals(cuda):
    mx, my = 16, 16
    rng = np.random.default_rng(0)
    q, aux = problem(2, mx, my, rng)
    L = _lib.lib()
    s = make_solver_struct(2, mx, my, 0.1, 0.1, [1, 1], [1, 1], [4] * 3, 2, 2, 0, PD[2],
                           capa=1)
    assert L.gclaw_check(ctypes.byref(s)) == _lib.ERR_ARG  # no aux array
    dev = DeviceProblem(s, aux=aux)
    s32 = make_solver_struct(2, mx, my, 0.1, 0.1, [1, 1], [1, 1], [4] * 3, 2, 2, 1, PD[2],
                             capa=1)
    s32.aux = dev.s.aux
    assert L.gclaw_check(ctypes.byref(s32)) == _lib.ERR_UNSUPPORTED  # FP64 only
    bad = make_solver_struct(2, mx, my, 0.1, 0.1, [1, 1], [1, 1], [4] * 3, 2, 2, 0, PD[2],
                             capa=2)
    bad.aux = dev.s.aux
    assert L.gclaw_check(ctypes.byref(bad)) == _lib.ERR_ARG  # kappa must follow the solver's aux
    with pytest.raises(_lib.GclawError):
        DeviceProblem(s, aux=aux, split=True).step(0.01)
    cfl = ctypes.c_double()
    assert L.gclaw_step2_noalloc(ctypes.byref(dev.s), None, None, 0.01, ctypes.byref(cfl),
                                 None) == _lib.ERR_UNSUPPORTED
    dev.upload(q)
    assert L.gclaw_adjoint_step(ctypes.byref(dev.s), ctypes.c_void_p(dev.q[0].data_ptr()),
                                ctypes.c_void_p(dev.q[0].data_ptr()),
                                ctypes.c_void_p(dev.q[1].data_ptr()), 0.01,
                                None) == _lib.ERR_UNSUPPORTED


def stretched_claw(mx=96, my=80, tfinal=0.3, nout=3):
    """Shallow-water dam break on a grid stretched in x: the computational
    cells are uniform and kappa is the physical cell width over dx."""
    x = pyclaw.Dimension(0.0, 1.0, mx, name="x")
    y = pyclaw.Dimension(0.0, 1.0, my, name="y")
    domain = pyclaw.Domain([x, y])
    state = pyclaw.State(domain, 3, 1)
    state.problem_data["grav"] = 1.0
    state.index_capa = 0
    X, Y = state.grid.p_centers
    state.aux[0] = 1.0 + 0.8 * np.exp(-20.0 * (X - 0.5) ** 2)
    state.q[0] = np.where((X - 0.4) ** 2 + (Y - 0.5) ** 2 < 0.04, 2.0, 1.0)
    state.q[1] = 0.0
    state.q[2] = 0.0
    solver = pyclaw.ClawSolver2D(riemann.shallow_roe_with_efix_2D)
    solver.dimensional_split = False
    solver.transverse_waves = 2
    solver.limiters = pyclaw.limiters.tvd.MC
    solver.bc_lower = [pyclaw.BC.wall, pyclaw.BC.wall]
    solver.bc_upper = [pyclaw.BC.wall, pyclaw.BC.wall]
    solver.aux_bc_lower = [pyclaw.BC.extrap, pyclaw.BC.extrap]
    solver.aux_bc_upper = [pyclaw.BC.extrap, pyclaw.BC.extrap]
    solver.dt_initial = 0.002
    claw = pyclaw.Controller()
    claw.solution = pyclaw.Solution(state, domain)
    claw.solver = solver
    claw.tfinal, claw.num_output_times = tfinal, nout
    return claw


def test_stretched_grid_through_pyclaw_front_end(cuda, oracle):
    claw = stretched_claw()
    q0 = claw.solution.state.q.copy()
    aux = claw.solution.state.aux.copy()
    dx, dy = claw.solution.state.grid.delta
    claw.run()
    assert len(claw.frames) == 4

    def step(q, dt):
        qn, cfl, rc = oracle.step_aux(2, [1.0], q, aux, dx, dy, dt, [3, 3], [3, 3], [1, 1],
                                      [1, 1], 2, 2, [4] * 3, nthreads=8, mcapa=1)
        assert rc == 0
        return qn, cfl

    q, t, dt = q0, 0.0, 0.002
    for k in range(1, 4):
        q, t, dt, _ = oracle.evolve(step, q, t, 0.1 * k, dt, cfl_desired=0.9, cfl_max=1.0)
        assert rel_l1(claw.frames[k].q, q) <= 1e-12, k
    # the physical mass, sum(kappa h), is conserved between walls
    m0 = (aux[0] * q0[0]).sum()
    assert abs((aux[0] * claw.frames[-1].q[0]).sum() - m0) <= 1e-12 * m0


@pytest.mark.parametrize("rp,capa", [(VC, False), (FW, False), (FW, True), (2, True)])
def test_f2py_shaped_step2_dropin_with_aux(cuda, oracle, rp, capa):
    """clawpack_gb300.classic2.step2 called as PyClaw calls the f2py module
    for solvers with aux, f-waves and a capacity (method[5] = mcapa)."""
    from clawpack_gb300 import classic2

    mod = {VC: riemann.vc_acoustics_2D, FW: riemann.shallow_bathymetry_fwave_2D,
           2: riemann.shallow_roe_with_efix_2D}[rp]
    if rp != VC:
        mod.cparam.grav = PD[rp][0]
    rng = np.random.default_rng(40 + rp + capa)
    mx, my = 33, 21
    q, aux = problem(rp, mx, my, rng)
    if not capa:
        aux = np.asfortranarray(aux[:-1])
    bcl, bcu = [1, 3], [1, 3]
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    auxbc = oracle.fill_aux_ghosts(aux, bcl, bcu)
    mcapa = aux.shape[0] if capa else 0
    method = np.array([1, 2, 2, 0, 1, mcapa, aux.shape[0]])
    mw = SHAPES[rp][1]
    out, cfl = classic2.step2(max(mx, my), 2, mx, my, qbc, qbc.copy(order="F"), auxbc, 0.05, 0.04,
                              0.001, method, [4] * mw, rp == FW, mod, mod)
    ref_q, ref_cfl, rc = oracle.step_aux(rp, PD[rp], q, aux, 0.05, 0.04, 0.001, bcl, bcu, bcl,
                                         bcu, 2, 2, [4] * 4, mcapa=mcapa)
    assert rel_l1(out[:, 2:-2, 2:-2], ref_q) <= 1e-13
    assert abs(cfl - ref_cfl) <= 1e-14 * ref_cfl
