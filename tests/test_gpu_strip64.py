"""The FP64 strip kernel (one warp per 28-column strip marching up its rows,
each row's accumulator starting from its state) against the oracle and the
FP64 tile kernel.

The strip kernel performs the oracle's IEEE operations in the oracle's
order, so the -fmad=false build (libgclaw_strict.so) reproduces the oracle
bit for bit; the product build agrees to 1e-13 relative L1 per step.
Ragged sizes exercise partial strips, several row segments and every
boundary mix."""
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
    def __init__(self, which, strict):
        self.which, self.strict = which, strict

    def __enter__(self):
        self.prev = _lib.lib(self.strict).gclaw_fp64_kernel(self.which)

    def __exit__(self, *exc):
        _lib.lib(self.strict).gclaw_fp64_kernel(self.prev)


def fp64_step(rp, q, dx, dy, dt, bcl, bcu, which, order=2, tw=2, lim=4, strict=True):
    s = make_solver_struct(rp, q.shape[1], q.shape[2], dx, dy, bcl, bcu, [lim] * SHAPES[rp][1],
                           order, tw, _lib.PREC_FP64, PD[rp])
    with kernel(which, strict):
        dev = DeviceProblem(s, strict=strict)
        dev.upload(q)
        dev.step(dt, src=0)
        c = dev.read_ctrl()
        return dev.download(1), c


SIZES = [(3, 70), (70, 3), (37, 29), (96, 40), (130, 77), (29, 200)]
BCS = [((1, 1), (1, 1)), ((2, 2), (2, 2)), ((3, 3), (3, 3)), ((3, 1), (1, 3))]


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("mx,my", SIZES)
@pytest.mark.parametrize("bcl,bcu", BCS)
def test_strict_strip_is_bitwise(cuda, oracle, rp, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx * 11 + my + 100 * rp)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.2 / my
    dt = 0.05 * min(dx, dy)
    lim = [1, 2, 3, 4][(mx + my) % 4]
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, bcl, bcu, 2, 2, [lim] * 4)
    qs, cs = fp64_step(rp, q, dx, dy, dt, bcl, bcu, STRIP, lim=lim)
    assert cs.status == 0
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert cs.cfl == cflo


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("order,tw,lim", [(2, 2, 4), (2, 1, 2), (2, 0, 3), (1, 1, 0), (1, 0, 0),
                                          (2, 2, 0), (2, 2, 1)])
def test_strict_strip_method_options(cuda, oracle, rp, order, tw, lim):
    mx, my = 45, 53
    rng = np.random.default_rng(5 + rp + 10 * order + tw)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, [3, 1], [1, 3], order, tw, [lim] * 4)
    qs, cs = fp64_step(rp, q, dx, dy, dt, [3, 1], [1, 3], STRIP, order, tw, lim)
    assert np.array_equal(qs, qo), np.abs(qs - qo).max()
    assert cs.cfl == cflo


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_product_strip_within_tolerance(cuda, oracle, rp):
    mx, my = 130, 77
    rng = np.random.default_rng(17 + rp)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, [2, 1], [2, 3], 2, 2, [4] * 4)
    qs, cs = fp64_step(rp, q, dx, dy, dt, [2, 1], [2, 3], STRIP, strict=False)
    assert cs.status == 0
    assert rel_l1(qs, qo) <= 1e-13, rel_l1(qs, qo)
    assert abs(cs.cfl - cflo) <= 1e-13 * cflo


@pytest.mark.parametrize("strict", [True, False])
def test_strip_step2_ghosted_input(cuda, oracle, strict):
    rp, mx, my = 2, 61, 47
    rng = np.random.default_rng(19)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    bcl, bcu = [3, 1], [1, 3]
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, bcl, bcu, 2, 2, [4] * 4)
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [4] * 3, 2, 2, _lib.PREC_FP64, PD[rp])
    L = _lib.lib(strict)
    with kernel(STRIP, strict):
        d_in = torch.from_numpy(np.ascontiguousarray(qbc.T)).cuda()
        d_out = d_in.clone()
        ws = torch.zeros(_lib.CTRL_BYTES, dtype=torch.uint8, device="cuda")
        cfl = ctypes.c_double()
        rc = L.gclaw_step2(ctypes.byref(s), ctypes.c_void_p(d_in.data_ptr()),
                           ctypes.c_void_p(d_out.data_ptr()), dt,
                           ctypes.c_void_p(ws.data_ptr()), ctypes.byref(cfl),
                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0
        qs = d_out.cpu().numpy().T
    assert np.array_equal(qs[:, :2, :], qbc[:, :2, :])  # ghosts untouched
    if strict:
        assert np.array_equal(qs[:, 2:-2, 2:-2], qo)
        assert cfl.value == cflo
    else:
        assert rel_l1(qs[:, 2:-2, 2:-2], qo) <= 1e-13


def test_strip_dam_break_run_matches_tile(cuda):
    """300 device-controlled steps of the 512^2 dam break in the strict
    build: the strip and tile kernels take the same steps to the same
    bits."""
    w = workloads.shallow_dam_break(512, 512)
    res = {}
    for which in (TILE, STRIP):
        with kernel(which, True):
            dev = DeviceProblem(w.solver_struct(_lib.PREC_FP64), strict=True)
            dev.upload(w.q0)
            c = dev.evolve(0.0, w.dt_initial, math.inf, max_accepted=300, max_steps=400)
            res[which] = (dev.download(c.parity), c)
    (qt, ct), (qs, cs) = res[TILE], res[STRIP]
    assert cs.numsteps == ct.numsteps == 300
    assert cs.t == ct.t
    assert np.array_equal(qs, qt)
