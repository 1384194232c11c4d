"""Batched launch of independent problems against single-problem runs.

Every problem of a batch runs the same body as a single problem (FP64: the
tile kernel; FP32-bulk: the strip kernel, or tiles when selected for the
process), so its state and its time-step control (t, dt, accepted and
attempted steps) must equal those of the same problem advanced alone, bit
for bit -- including problems whose first dt is rejected."""
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, workloads
from clawpack_gb300.batch import BatchSolver
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import rel_l1

pytestmark = pytest.mark.gpu


def small_batch(nprob, seed, precision):
    rng = np.random.default_rng(seed)
    shapes = [(int(rng.integers(3, 90)), int(rng.integers(3, 90))) for _ in range(nprob)]
    deltas = [(1.0 / mx, 1.3 / my) for mx, my in shapes]
    qs, dt0 = [], []
    for p, (mx, my) in enumerate(shapes):
        q = np.zeros((3, mx, my), order="F")
        q[0] = 1.0 + 0.5 * rng.random((mx, my))
        q[1] = 0.3 * rng.normal(size=(mx, my))
        q[2] = 0.3 * rng.normal(size=(mx, my))
        qs.append(q)
        dx = min(deltas[p])
        dt0.append(0.4 * dx if p % 5 else 10.0 * dx)  # every 5th problem starts with a rejection
    bs = BatchSolver(_lib.RP_SHALLOW_ROE_WITH_EFIX_2D, shapes, deltas, [3, 1], [1, 3], [4, 4, 4],
                     [1.0], precision=precision)
    host = bs.pinned_host_buffer()
    for p, q in enumerate(qs):
        bs.pack(host, p, q)
    bs.upload(host)
    return bs, shapes, deltas, qs, np.array(dt0)


@pytest.mark.parametrize("precision,family", [(_lib.PREC_FP64, 0), (_lib.PREC_FP32_BULK, 0),
                                              (_lib.PREC_FP32_BULK, 1)])
def test_batch_equals_single_problems(cuda, precision, family):
    nsteps = 12
    prev = _lib.lib().gclaw_fp32_kernel(family)  # 0: default (strips), 1: tiles
    try:
        _batch_equals_single_problems(precision, nsteps)
    finally:
        _lib.lib().gclaw_fp32_kernel(prev)


def _batch_equals_single_problems(precision, nsteps):
    bs, shapes, deltas, qs, dt0 = small_batch(24, 7 + precision, precision)
    bs.ctrl_init(dt0, max_accepted=nsteps, max_steps=100)
    for _ in range(4 * nsteps):
        bs.advance(1)
    ctrl = bs.read_ctrls()
    outs = bs.download()
    assert np.all(ctrl["done"] == 1) and np.all(ctrl["status"] == 0)
    assert np.all(ctrl["numsteps"] == nsteps)
    assert np.any(ctrl["attempts"] > nsteps)  # the rejected first attempts
    singles = []
    for p, ((mx, my), (dx, dy)) in enumerate(zip(shapes, deltas)):
        s = make_solver_struct(_lib.RP_SHALLOW_ROE_WITH_EFIX_2D, mx, my, dx, dy, [3, 1],
                               [1, 3], [4, 4, 4], 2, 2, precision, [1.0])
        dev = DeviceProblem(s)
        dev.upload(qs[p])
        c = dev.evolve(0.0, dt0[p], math.inf, max_accepted=nsteps, max_steps=100)
        singles.append((dev.download(c.parity), c))
    for p, (q1, c) in enumerate(singles):
        assert np.array_equal(q1, outs[p]), p
        assert (c.t, c.dt, c.numsteps, c.attempts) == (ctrl["t"][p], ctrl["dt"][p],
                                                       ctrl["numsteps"][p], ctrl["attempts"][p])


def test_batch_graph_capture_matches_eager(cuda):
    bs, shapes, deltas, qs, dt0 = small_batch(16, 3, _lib.PREC_FP32_BULK)
    bs.ctrl_init(dt0, max_accepted=9, max_steps=100)
    bs.advance(20)
    eager = bs.download()
    bs2, *_ = small_batch(16, 3, _lib.PREC_FP32_BULK)
    g = bs2.capture(5)
    bs2.ctrl_init(dt0, max_accepted=9, max_steps=100)
    for _ in range(4):
        g.replay()
    torch.cuda.synchronize()
    for a, b in zip(eager, bs2.download()):
        assert np.array_equal(a, b)


def test_full_ensemble_steps_conserve_mass(cuda):
    """All 4096 problems (193 M cells) for 10 FP32-bulk steps: every problem
    advances, wall boundaries conserve each problem's mass."""
    e = workloads.batched_ensemble(nsteps=10)
    bs = workloads.make_batch(e)
    for _ in range(10):
        bs.advance(1)
    ctrl = bs.read_ctrls()
    assert np.all(ctrl["status"] == 0) and np.all(ctrl["numsteps"] == 10)
    outs = bs.download()
    for p in range(0, len(outs), 97):
        m0 = e.q0(p)[0].sum()
        assert abs(outs[p][0].sum() - m0) <= 2e-7 * m0, p


def test_ensemble_fp32_within_1e5_of_fp64(cuda):
    """200 steps of the first 128 ensemble problems: FP32-bulk vs FP64."""
    e = workloads.batched_ensemble(nsteps=200)
    e.shapes, e.deltas, e.params, e.dt0 = e.shapes[:128], e.deltas[:128], e.params[:128], e.dt0[:128]
    res = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_FP32_BULK):
        bs = workloads.make_batch(e, precision=prec)
        bs.advance(210)
        assert np.all(bs.read_ctrls()["numsteps"] == 200)
        res[prec] = bs.download()
    errs = [rel_l1(a, b) for a, b in zip(res[_lib.PREC_FP32_BULK], res[_lib.PREC_FP64])]
    assert max(errs) <= 1e-5, max(errs)
