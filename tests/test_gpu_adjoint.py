"""The hand-written adjoint kernel and the checkpointed autograd Function.

One step: lam^T (d step / d q) from gclaw_adjoint_step against torch.autograd
through the PyTorch transcription of the step (oracle/classic2_torch.py),
in FP64 (the -fmad=false build agrees to 1e-11 relative, the product build
to 1e-10) and in FP32 (1e-4).  Whole runs: the gradient of the gauge
least-squares loss from EvolveGauges (checkpointing + recomputation +
reverse adjoint steps) against torch autograd through the transcription and
against central finite differences of the FP64 forward at the same fixed dt
sequence."""
import ctypes

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, adjoint, workloads
from clawpack_gb300.device import make_solver_struct
from oracle import classic2_torch as ct
from tests.helpers import PD, SHAPES, random_state

pytestmark = pytest.mark.gpu


def cuda_vjp(rp, q, lam, dx, dy, dt, bcl, bcu, lim, order, tw, precision=0, strict=False):
    mw = SHAPES[rp][1]
    s = make_solver_struct(rp, q.shape[1], q.shape[2], dx, dy, bcl, bcu, [lim] * mw, order, tw,
                           precision, PD[rp])
    L = _lib.lib(strict)
    dq = torch.from_numpy(np.ascontiguousarray(q.T)).cuda()
    dl = torch.from_numpy(np.ascontiguousarray(lam.T)).cuda()
    out = torch.empty_like(dl)
    rc = L.gclaw_adjoint_step(ctypes.byref(s), ctypes.c_void_p(dq.data_ptr()),
                              ctypes.c_void_p(dl.data_ptr()), ctypes.c_void_p(out.data_ptr()), dt,
                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().T


def torch_vjp(rp, q, lam, dx, dy, dt, bcl, bcu, lim, order, tw):
    qt = torch.from_numpy(np.ascontiguousarray(q)).requires_grad_(True)
    qn, _ = ct.step(rp, PD[rp], qt, dx, dy, dt, bcl, bcu, order, tw, [lim] * 4)
    (qn * torch.from_numpy(np.ascontiguousarray(lam))).sum().backward()
    return qt.grad.numpy()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


CASES = [(rp, mx, my, bcl, bcu, lim, order, tw)
         for rp in (1, 2)
         for (mx, my) in ((37, 29), (16, 16), (9, 40))
         for (bcl, bcu) in (([1, 1], [1, 1]), ([3, 3], [3, 3]), ([2, 3], [2, 1]))
         for (lim, order, tw) in ((4, 2, 2), (2, 2, 1), (1, 1, 0), (0, 2, 2))]


@pytest.mark.parametrize("rp,mx,my,bcl,bcu,lim,order,tw", CASES)
def test_adjoint_step_matches_torch_autograd(cuda, rp, mx, my, bcl, bcu, lim, order, tw):
    rng = np.random.default_rng(mx * 31 + my + 7 * rp + lim)
    q = random_state(rp, mx, my, rng)
    lam = rng.normal(size=q.shape)
    dx, dy, dt = 1.0 / mx, 1.2 / my, 0.1 / max(mx, my)
    ref = torch_vjp(rp, q, lam, dx, dy, dt, bcl, bcu, lim, order, tw)
    strict = cuda_vjp(rp, q, lam, dx, dy, dt, bcl, bcu, lim, order, tw, strict=True)
    assert rel(strict, ref) <= 1e-11
    prod = cuda_vjp(rp, q, lam, dx, dy, dt, bcl, bcu, lim, order, tw)
    assert rel(prod, ref) <= 1e-10
    f32 = cuda_vjp(rp, q, lam, dx, dy, dt, bcl, bcu, lim, order, tw, precision=1)
    assert rel(f32, ref) <= 1e-4


def loss_of(series, target):
    return ((series - target) ** 2).sum()


def gauge_setup(p):
    """Fixed dt sequence (FP64 CFL rule on the undisturbed run), gauges and
    target series of the problem."""
    dev = torch.device("cuda")
    s64 = p.solver_struct(_lib.PREC_FP64)
    dts = adjoint.record_dts(torch.from_numpy(p.q0()).to(dev), s64, p.nsteps, p.dt0)
    gauges = torch.as_tensor(p.gauges, device=dev)
    target = adjoint.gauge_series(torch.from_numpy(p.q0(p.h_true)).to(dev), s64, dts, gauges)
    return dts, gauges, target


def cuda_gradient(p, dts, gauges, target, precision=_lib.PREC_FP64):
    h0 = torch.from_numpy(p.h0).cuda().requires_grad_(True)
    q = torch.stack([h0, torch.zeros_like(h0), torch.zeros_like(h0)])
    L = loss_of(adjoint.evolve_gauges(q, p.solver_struct(precision), dts, gauges,
                                      p.checkpoint_every), target)
    L.backward()
    return float(L.detach()), h0.grad.cpu().numpy()


def central_fd(p, dts, gauges, target, v, eps):
    """Central difference of the FP64 loss along v at the same fixed dts."""
    s64 = p.solver_struct(_lib.PREC_FP64)
    vals = []
    for sgn in (1, -1):
        qq = torch.from_numpy(p.q0(p.h0 + sgn * eps * v)).cuda()
        vals.append(float(loss_of(adjoint.gauge_series(qq, s64, dts, gauges), target)))
    return (vals[0] - vals[1]) / (2 * eps)


def smooth_directions(p, n, seed):
    """Gaussian perturbations exp(-80 |x - c|^2) centred in the domain.  A
    white-noise direction of size eps puts waves of size eps into the flat
    far field, where the undisturbed waves are at roundoff level, and flips
    limiter branches there; along smooth directions the loss is
    differentiable at the step sizes used."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.linspace(0, 1, p.mx), np.linspace(0, 1, p.my), indexing="ij")
    for _ in range(n):
        c = rng.uniform(0.2, 0.8, 2)
        yield np.exp(-80.0 * ((X - c[0]) ** 2 + (Y - c[1]) ** 2))


def test_checkpointed_gradient_matches_torch_autograd_and_fd(cuda):
    """40x36, 30 steps, MC limiter, checkpoints every 7 steps; 64 gauges, some
    of them in the same cell."""
    p = workloads.adjoint_problem(40, 36, nsteps=30, checkpoint_every=7)
    assert len({tuple(g) for g in p.gauges}) < len(p.gauges)  # duplicate gauges exercised
    dts, gauges, target = gauge_setup(p)
    L, g_cuda = cuda_gradient(p, dts, gauges, target)
    # torch autograd through the transcription (CPU, FP64)
    h0t = torch.from_numpy(p.h0.copy()).requires_grad_(True)
    qt = torch.stack([h0t, torch.zeros_like(h0t), torch.zeros_like(h0t)])
    series = []
    gx, gy = p.gauges[:, 0], p.gauges[:, 1]
    for dt in dts:
        qt, _ = ct.step(2, [1.0], qt, p.dx, 1.0 / p.my, dt, [3, 3], [3, 3], 2, 2, [4] * 4)
        series.append(qt[0, gx, gy])
    Lt = loss_of(torch.stack(series), target.cpu())
    Lt.backward()
    assert abs(L - float(Lt.detach())) <= 1e-12 * float(Lt.detach())
    assert rel(g_cuda, h0t.grad.numpy()) <= 1e-9
    for v in smooth_directions(p, 2, 2):
        fd = central_fd(p, dts, gauges, target, v, 1e-7)
        ad = float((g_cuda * v).sum())
        assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_unlimited_gradient_matches_fd_in_every_direction(cuda):
    """Unlimited Lax-Wendroff corrections (limiter 0) on a subsonic flow make
    the discrete map smooth, so central differences along white-noise
    directions agree with the adjoint, in FP64 and in FP32-bulk."""
    p = workloads.adjoint_problem(40, 36, nsteps=30, checkpoint_every=7, limiter=0)
    dts, gauges, target = gauge_setup(p)
    _, g64 = cuda_gradient(p, dts, gauges, target)
    _, g32 = cuda_gradient(p, dts, gauges, target, _lib.PREC_FP32_BULK)
    rng = np.random.default_rng(3)
    for _ in range(2):
        v = rng.normal(size=p.h0.shape)
        fd = central_fd(p, dts, gauges, target, v, 1e-6)
        assert abs(float((g64 * v).sum()) - fd) <= 1e-6 * abs(fd)
        assert abs(float((g32 * v).sum()) - fd) <= 1e-5 * abs(fd)


def test_adjoint_problem_full_size_fp32_gradient_vs_fp64_fd(cuda):
    """1024^2, 500 steps, MC limiter, checkpoints every 23 steps: the FP64 and
    the FP32-bulk gradients against FP64 central finite differences (fixed
    dts) along smooth directions."""
    p = workloads.adjoint_problem()
    dts, gauges, target = gauge_setup(p)
    _, g64 = cuda_gradient(p, dts, gauges, target)
    _, g32 = cuda_gradient(p, dts, gauges, target, _lib.PREC_FP32_BULK)
    for v in smooth_directions(p, 2, 2):
        fd = central_fd(p, dts, gauges, target, v, 1e-6)
        assert abs(float((g64 * v).sum()) - fd) <= 1e-6 * abs(fd)
        assert abs(float((g32 * v).sum()) - fd) <= 1e-5 * abs(fd)
