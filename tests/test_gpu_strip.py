"""The FP32-bulk strip kernel (one warp per 28-column strip marching up its
rows) against the FP32-bulk tile kernel and the oracle.

Both kernels evaluate the same per-edge functions in the same accumulation
order, so they agree to rounding of multiply-add contraction (1e-6
relative); ragged sizes exercise partial strips, several row segments and
every boundary mix, including ghost-filled qbc input (gclaw_step2)."""
import ctypes
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, workloads
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import PD, SHAPES, random_state, rel_l1

pytestmark = pytest.mark.gpu

TILE, STRIP = 1, 2


class kernel:
    def __init__(self, which):
        self.which = which

    def __enter__(self):
        self.prev = _lib.lib().gclaw_fp32_kernel(self.which)

    def __exit__(self, *exc):
        _lib.lib().gclaw_fp32_kernel(self.prev)


def fp32_step(rp, q, dx, dy, dt, bcl, bcu, which, order=2, tw=2, lim=4):
    s = make_solver_struct(rp, q.shape[1], q.shape[2], dx, dy, bcl, bcu, [lim] * SHAPES[rp][1],
                           order, tw, _lib.PREC_FP32_BULK, PD[rp])
    with kernel(which):
        dev = DeviceProblem(s)
        dev.upload(q)
        dev.step(dt, src=0)
        c = dev.read_ctrl()
        return dev.download(1), c


SIZES = [(3, 70), (70, 3), (37, 29), (96, 40), (130, 77), (29, 200)]
BCS = [((1, 1), (1, 1)), ((2, 2), (2, 2)), ((3, 3), (3, 3)), ((3, 1), (1, 3))]


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("mx,my", SIZES)
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_strip_equals_tile(cuda, rp, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx * 7 + my + 100 * rp)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.2 / my
    dt = 0.05 * min(dx, dy)
    lim = [1, 2, 3, 4][(mx + my) % 4]
    qt, ct = fp32_step(rp, q, dx, dy, dt, bcl, bcu, TILE, lim=lim)
    qs, cs = fp32_step(rp, q, dx, dy, dt, bcl, bcu, STRIP, lim=lim)
    assert cs.status == ct.status == 0
    assert rel_l1(qs, qt) <= 1e-6, rel_l1(qs, qt)
    assert abs(cs.cfl - ct.cfl) <= 1e-6 * ct.cfl


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("order,tw,lim", [(2, 2, 4), (2, 1, 2), (2, 0, 3), (1, 1, 0), (1, 0, 0),
                                          (2, 2, 0)])
def test_strip_method_options_against_oracle(cuda, oracle, rp, order, tw, lim):
    mx, my = 45, 53
    rng = np.random.default_rng(3 + rp + 10 * order + tw)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, [3, 1], [1, 3], order, tw, [lim] * 4)
    qs, cs = fp32_step(rp, q, dx, dy, dt, [3, 1], [1, 3], STRIP, order, tw, lim)
    assert rel_l1(qs, qo) <= 2e-6
    assert abs(cs.cfl - cflo) <= 1e-5 * cflo


def test_strip_step2_ghosted_input(cuda, oracle):
    rp, mx, my = 2, 61, 47
    rng = np.random.default_rng(9)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    bcl, bcu = [3, 1], [1, 3]
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [4] * 3, 2, 2, _lib.PREC_FP32_BULK,
                           PD[rp])
    L = _lib.lib()
    outs = {}
    for which in (TILE, STRIP):
        with kernel(which):
            d_in = torch.from_numpy(np.ascontiguousarray(qbc.T)).cuda()
            d_out = d_in.clone()
            ws = torch.zeros(_lib.CTRL_BYTES, dtype=torch.uint8, device="cuda")
            cfl = ctypes.c_double()
            rc = L.gclaw_step2(ctypes.byref(s), ctypes.c_void_p(d_in.data_ptr()),
                               ctypes.c_void_p(d_out.data_ptr()), dt,
                               ctypes.c_void_p(ws.data_ptr()), ctypes.byref(cfl),
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
            assert rc == 0
            outs[which] = (d_out.cpu().numpy().T, cfl.value)
    (qt, ct), (qs, cs) = outs[TILE], outs[STRIP]
    assert rel_l1(qs[:, 2:-2, 2:-2], qt[:, 2:-2, 2:-2]) <= 1e-6
    assert np.array_equal(qs[:, :2, :], qbc[:, :2, :])  # ghosts untouched
    assert abs(cs - ct) <= 1e-6 * ct


def test_strip_dam_break_run_matches_tile(cuda):
    """300 device-controlled steps of the 512^2 dam break: same step count,
    same time and states within 1e-6."""
    w = workloads.shallow_dam_break(512, 512)
    res = {}
    for which in (TILE, STRIP):
        with kernel(which):
            dev = DeviceProblem(w.solver_struct(_lib.PREC_FP32_BULK))
            dev.upload(w.q0)
            c = dev.evolve(0.0, w.dt_initial, math.inf, max_accepted=300, max_steps=400)
            res[which] = (dev.download(c.parity), c)
    (qt, ct), (qs, cs) = res[TILE], res[STRIP]
    assert cs.numsteps == ct.numsteps == 300
    assert abs(cs.t - ct.t) <= 1e-6 * ct.t
    assert rel_l1(qs, qt) <= 1e-6
