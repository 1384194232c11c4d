"""Parity of the CUDA step (through the C ABI) with the CPU oracle.

Tolerances: the -fmad=false build (libgclaw_strict.so) must reproduce the
oracle bit for bit, because it performs the same IEEE operations in the same
order; the product build (FMA contraction on) must agree to 1e-13 relative
L1 per step; the FP32-bulk mode to 2e-6 relative L1 per step."""
import ctypes

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib
from clawpack_gb300.device import DeviceProblem, make_solver_struct
from tests.helpers import PD, SHAPES, random_state, rel_l1

pytestmark = pytest.mark.gpu

SIZES = [(2, 2), (3, 70), (70, 3), (37, 29), (33, 9), (65, 17), (96, 40)]
BCS = [((1, 1), (1, 1)), ((2, 2), (2, 2)), ((3, 3), (3, 3)), ((3, 1), (1, 3))]


def gpu_step(rp, q, dx, dy, dt, bcl, bcu, order=2, tw=2, lim=4, precision=0, strict=False):
    mw = SHAPES[rp][1]
    s = make_solver_struct(rp, q.shape[1], q.shape[2], dx, dy, bcl, bcu, [lim] * mw, order, tw,
                           precision, PD[rp])
    dev = DeviceProblem(s, strict=strict)
    dev.upload(q)
    dev.step(dt, src=0)
    c = dev.read_ctrl()
    return dev.download(1), c


def cases():
    out = []
    for rp in (1, 2, 3):
        for (mx, my) in SIZES:
            for bcl, bcu in BCS:
                out.append((rp, mx, my, bcl, bcu))
    return out


@pytest.mark.parametrize("rp,mx,my,bcl,bcu", cases())
def test_strict_build_is_bitwise(cuda, oracle, rp, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx * 1000 + my + rp)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.3 / my
    dt = 0.05 * min(dx, dy)
    lim = [1, 2, 3, 4][(mx + my) % 4]
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, bcl, bcu, 2, 2, [lim] * 4)
    qg, c = gpu_step(rp, q, dx, dy, dt, bcl, bcu, 2, 2, lim, strict=True)
    assert c.status == 0
    assert np.array_equal(qg, qo), np.abs(qg - qo).max()
    assert c.cfl == cflo


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("order,tw", [(2, 2), (2, 1), (2, 0), (1, 1), (1, 0)])
@pytest.mark.parametrize("lim", [0, 1, 2, 3, 4])
def test_strict_all_method_options(cuda, oracle, rp, order, tw, lim):
    rng = np.random.default_rng(7 * rp + 11 * order + 13 * tw + lim)
    q = random_state(rp, 41, 35, rng)
    dx = dy = 0.05
    dt = 0.004
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, [3, 1], [1, 3], order, tw, [lim] * 4)
    qg, c = gpu_step(rp, q, dx, dy, dt, [3, 1], [1, 3], order, tw, lim, strict=True)
    assert np.array_equal(qg, qo)
    assert c.cfl == cflo


@pytest.mark.parametrize("rp,mx,my,bcl,bcu", cases()[::3])
def test_product_build_within_tolerance(cuda, oracle, rp, mx, my, bcl, bcu):
    rng = np.random.default_rng(mx + 17 * my + rp)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    dt = 0.05 * min(dx, dy)
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, bcl, bcu, 2, 2, [4] * 4)
    qg, c = gpu_step(rp, q, dx, dy, dt, bcl, bcu, 2, 2, 4)
    assert rel_l1(qg, qo) <= 1e-13
    assert abs(c.cfl - cflo) <= 1e-14 * cflo


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_fp32_bulk_single_step(cuda, oracle, rp):
    rng = np.random.default_rng(100 + rp)
    q = random_state(rp, 90, 70, rng)
    dx = dy = 0.02
    dt = 0.0015
    qo, cflo, rc = oracle.step(rp, PD[rp], q, dx, dy, dt, [1, 1], [1, 1], 2, 2, [4] * 4)
    qg, c = gpu_step(rp, q, dx, dy, dt, [1, 1], [1, 1], 2, 2, 4, precision=1)
    assert rel_l1(qg, qo) <= 2e-6
    assert abs(c.cfl - cflo) <= 1e-5 * cflo


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_step2_dropin_matches_fused_boundary_path(cuda, oracle, rp):
    """gclaw_step2 on an oracle-filled qbc equals gclaw_step with on-device
    boundary conditions, bit for bit, and leaves qnew's ghosts untouched."""
    rng = np.random.default_rng(200 + rp)
    mx, my = 45, 38
    q = random_state(rp, mx, my, rng)
    dx, dy, dt = 0.03, 0.02, 0.001
    bcl, bcu = [3, 2], [1, 2]
    mw = SHAPES[rp][1]
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [2] * mw, 2, 2, 0, PD[rp])
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    d_old = torch.from_numpy(np.ascontiguousarray(qbc.T)).cuda()
    d_new = torch.full_like(d_old, -7.0)
    ws = torch.zeros(256, dtype=torch.uint8, device="cuda")
    cfl = ctypes.c_double()
    L = _lib.lib()
    rc = L.gclaw_step2(ctypes.byref(s), ctypes.c_void_p(d_old.data_ptr()),
                       ctypes.c_void_p(d_new.data_ptr()), dt, ctypes.c_void_p(ws.data_ptr()),
                       ctypes.byref(cfl), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    new = np.asfortranarray(d_new.cpu().numpy().T)
    qg, c = gpu_step(rp, q, dx, dy, dt, bcl, bcu, 2, 2, 2)
    assert np.array_equal(new[:, 2:-2, 2:-2], qg)
    assert cfl.value == c.cfl
    ghost = np.ones(new.shape, bool)
    ghost[:, 2:-2, 2:-2] = False
    assert np.all(new[ghost] == -7.0)


def test_nan_state_reports_nonphysical(cuda):
    rng = np.random.default_rng(5)
    q = random_state(2, 20, 20, rng)
    q[0, 7, 9] = np.nan
    qg, c = gpu_step(2, q, 0.05, 0.05, 0.001, [1, 1], [1, 1])
    assert c.status == _lib.NONPHYSICAL


def test_negative_pressure_reports_nonphysical(cuda):
    rng = np.random.default_rng(6)
    q = random_state(3, 20, 20, rng)
    q[3, 4, 4] = 0.01 * q[3, 4, 4] - 10.0  # E so low that the Roe c^2 < 0
    qg, c = gpu_step(3, q, 0.05, 0.05, 0.001, [1, 1], [1, 1])
    assert c.status == _lib.NONPHYSICAL


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_f2py_shaped_step2_dropin(cuda, oracle, rp):
    """clawpack_gb300.classic2.step2 called exactly as PyClaw calls the f2py
    classic2.step2, with numpy qbc arrays and the riemann module's cparam."""
    from clawpack_gb300 import classic2, riemann

    mod = {1: riemann.acoustics_2D, 2: riemann.shallow_roe_with_efix_2D,
           3: riemann.euler_4wave_2D}[rp]
    names = {1: dict(rho=1.0, bulk=4.0, cc=2.0, zz=2.0), 2: dict(grav=1.0),
             3: dict(gamma=1.4, efix=True)}[rp]
    for k, v in names.items():
        setattr(mod.cparam, k, v)
    rng = np.random.default_rng(300 + rp)
    mx, my = 33, 21
    q = random_state(rp, mx, my, rng)
    qbc = oracle.fill_ghosts(q, [1, 3], [1, 3])
    qnew = qbc.copy(order="F")
    method = np.array([1, 2, 2, 0, 1, 0, 0])
    mw = SHAPES[rp][1]
    out, cfl = classic2.step2(max(mx, my), 2, mx, my, qbc, qnew, None, 0.05, 0.04, 0.002, method,
                              [4] * mw, False, mod, mod)
    ref_q, ref_cfl = oracle.step2(rp, PD[rp], qbc, 0.05, 0.04, 0.002, 2, 2, [4] * 4)
    assert out is qnew
    assert rel_l1(out[:, 2:-2, 2:-2], ref_q[:, 2:-2, 2:-2]) <= 1e-13
    assert abs(cfl - ref_cfl) <= 1e-14 * ref_cfl
