"""Dimensionally split steps on the GPU (gclaw_step_split /
gclaw_advance_split, ClawSolver2D with dimensional_split=True) against the
oracle's split step.

The -fmad=false build must reproduce the oracle bit for bit, single steps
and whole controlled runs including a rejected first attempt; the product
build within 1e-13 relative L1 per step, FP32-bulk within 2e-6."""
import ctypes
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, pyclaw, workloads
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import PD, SHAPES, random_state, rel_l1

pytestmark = pytest.mark.gpu

SIZES = [(2, 2), (3, 70), (37, 29), (96, 40), (250, 3), (131, 17)]
BCS = [((1, 1), (1, 1)), ((2, 2), (2, 2)), ((3, 3), (3, 3)), ((3, 1), (1, 3))]


def split_struct(rp, mx, my, dx, dy, bcl, bcu, lim, order=2, precision=0):
    return make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [lim] * SHAPES[rp][1], order, 2,
                              precision, PD[rp])


def gpu_split_step(s, q, dt, strict=False):
    dev = DeviceProblem(s, strict=strict, split=True)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("mx,my", SIZES)
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_split_step_strict_is_bitwise(cuda, oracle, rp, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx * 100 + my + rp)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.3 / my
    dt = 0.05 * min(dx, dy)
    lim = [1, 2, 3, 4][(mx + my) % 4]
    qo, cflo, rc = oracle.step_split(rp, PD[rp], q, dx, dy, dt, bcl, bcu, 2, [lim] * 4)
    assert rc == 0
    s = split_struct(rp, mx, my, dx, dy, bcl, bcu, lim)
    qs, c = gpu_split_step(s, q, dt, strict=True)
    assert c.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert c.cfl == cflo
    qp, cp = gpu_split_step(s, q, dt)
    assert rel_l1(qp, qo) <= 1e-13 and abs(cp.cfl - cflo) <= 1e-14 * cflo
    s32 = split_struct(rp, mx, my, dx, dy, bcl, bcu, lim, precision=_lib.PREC_FP32_BULK)
    q32, c32 = gpu_split_step(s32, q, dt)
    assert rel_l1(q32, qo) <= 2e-6 and abs(c32.cfl - cflo) <= 1e-5 * cflo


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("order", [1, 2])
def test_split_order_and_limiters(cuda, oracle, rp, order):
    mx, my = 41, 33
    rng = np.random.default_rng(5 + rp + order)
    q = random_state(rp, mx, my, rng)
    dx, dy, dt = 1.0 / mx, 1.0 / my, 0.04 / max(mx, my)
    for lim in (0, 1, 2, 3, 4):
        qo, cflo, _ = oracle.step_split(rp, PD[rp], q, dx, dy, dt, [3, 1], [1, 3], order,
                                        [lim] * 4)
        qs, c = gpu_split_step(split_struct(rp, mx, my, dx, dy, [3, 1], [1, 3], lim, order), q,
                               dt, strict=True)
        assert np.array_equal(qs, qo), lim
        assert c.cfl == cflo


def test_split_controlled_run_with_rejection_is_bitwise(cuda, oracle):
    """The 128^2 dam break for 60 split steps under device control, starting
    with a dt that is rejected: the same attempts, steps, times and state."""
    w = workloads.shallow_dam_break(128, 128)
    mw = 3

    def step(q, dt):
        qn, cfl, rc = oracle.step_split(w.rp_id, w.pd_array(), q, w.dx, w.dy, dt, w.bc_lower,
                                        w.bc_upper, w.order, w.mthlim(mw), nthreads=8)
        assert rc == 0
        return qn, cfl

    dt0 = 5.0 * w.dt_initial
    qo, to, dto, st = oracle.evolve(step, w.q0, 0.0, math.inf, dt0, cfl_desired=w.cfl_desired,
                                    cfl_max=w.cfl_max, max_accepted=60)
    assert st["attempts"] > st["numsteps"] == 60
    dev = DeviceProblem(w.solver_struct(0), strict=True, split=True)
    dev.upload(w.q0)
    c = dev.evolve(0.0, dt0, math.inf, cfl_max=w.cfl_max, cfl_desired=w.cfl_desired,
                   max_accepted=60, max_steps=200)
    assert (c.numsteps, c.attempts) == (st["numsteps"], st["attempts"])
    assert c.t == to and c.dt == dto
    assert np.array_equal(dev.download(c.parity), qo)


def test_default_solver_is_split_and_runs(cuda, oracle):
    """ClawSolver2D's default (dimensional_split=True) runs the acoustics
    problem through the Controller: the last frame matches the oracle's split
    evolve within 1e-12 (product build), host and device control agree."""
    w = workloads.acoustics_radial(80, 80)
    w.tfinal, w.num_output_times = 0.2, 2
    outs = []
    for dc in (True, False):
        claw = workloads.make_claw(w)
        claw.solver.dimensional_split = True
        claw.solver.device_control = dc
        claw.run()
        outs.append(claw.frames[-1].q)
    assert np.array_equal(outs[0], outs[1])

    def step(q, dt):
        qn, cfl, rc = oracle.step_split(w.rp_id, w.pd_array(), q, w.dx, w.dy, dt, w.bc_lower,
                                        w.bc_upper, w.order, w.mthlim(2), nthreads=8)
        return qn, cfl

    q, t, dt = w.q0, 0.0, w.dt_initial
    for tout in (0.1, 0.2):
        q, t, dt, _ = oracle.evolve(step, q, t, tout, dt, cfl_desired=w.cfl_desired,
                                    cfl_max=w.cfl_max)
    assert rel_l1(outs[0], q) <= 1e-12
    assert pyclaw.ClawSolver2D(None).dimensional_split is True


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("precision", [0, 1])
def test_split_kernel_families_agree(cuda, rp, precision):
    """The kernel families of the split step -- the default, the tile kernels
    with a sweep mask (gclaw_split_kernel(1)), marching columns for the
    y-sweep (2) and warp windows for both sweeps (3) -- give bit-identical
    steps in the strict build, on a grid of several warp windows and column
    chunks."""
    mx, my = 300, 251
    rng = np.random.default_rng(rp + 10 * precision)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    s = split_struct(rp, mx, my, dx, dy, (3, 2), (1, 2), 4, precision=precision)
    L = _lib.lib(True)
    res = {}
    for fam in (1, 2, 3, 0):
        prev = L.gclaw_split_kernel(fam)
        try:
            res[fam] = gpu_split_step(s, q, 0.04 * min(dx, dy), strict=True)
        finally:
            L.gclaw_split_kernel(prev)
    for fam in (1, 2, 3):
        assert np.array_equal(res[fam][0], res[0][0]), fam
        assert res[fam][1].cfl == res[0][1].cfl and res[fam][1].status == res[0][1].status == 0
