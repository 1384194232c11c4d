"""Time-stepping on the GPU against the oracle's evolve_to_time loop.

The acoustics problem runs at its full size (200x200, t_final 0.6, 10
frames): the strict build must reproduce every frame bit for bit with the
same accepted/rejected attempts; the product build must stay within 1e-12
relative L1 at every frame.  The shallow-water and Euler problems run at
reduced sizes against the oracle, and at full size through size-independent
properties (conservation, symmetry, FP32 error bound)."""
import ctypes
import math

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib, workloads
from clawpack_gb300.device import DeviceProblem
from tests.helpers import rel_l1

pytestmark = pytest.mark.gpu


def struct_of(w, precision=0):
    return w.solver_struct(precision)


def oracle_frames(oracle, w, nthreads=8):
    mw = {1: 2, 2: 3, 3: 4}[w.rp_id]

    def step(q, dt):
        qn, cfl, rc = oracle.step(w.rp_id, w.pd_array(), q, w.dx, w.dy, dt, w.bc_lower,
                                  w.bc_upper, w.order, w.transverse_waves, w.mthlim(mw),
                                  nthreads=nthreads)
        assert rc == 0
        return qn, cfl

    q, t, dt = w.q0, 0.0, w.dt_initial
    frames, logs = [q], []
    if w.tfinal is not None:
        for tout in np.linspace(0.0, w.tfinal, w.num_output_times + 1)[1:]:
            q, t, dt, st = oracle.evolve(step, q, t, tout, dt, cfl_desired=w.cfl_desired,
                                         cfl_max=w.cfl_max)
            frames.append(q)
            logs.append(st)
    else:
        q, t, dt, st = oracle.evolve(step, q, t, math.inf, dt, cfl_desired=w.cfl_desired,
                                     cfl_max=w.cfl_max, max_accepted=w.nsteps)
        frames.append(q)
        logs.append(st)
    return frames, logs


def device_frames(w, strict=False, precision=0, device_control=True):
    dev = DeviceProblem(struct_of(w, precision), strict=strict)
    dev.upload(w.q0)
    t, dt = 0.0, w.dt_initial
    frames, ctrls = [w.q0], []
    touts = (np.linspace(0.0, w.tfinal, w.num_output_times + 1)[1:] if w.tfinal is not None
             else [math.inf])
    for tout in touts:
        c = dev.evolve(t, dt, tout, cfl_max=w.cfl_max, cfl_desired=w.cfl_desired,
                       max_accepted=-1 if w.tfinal is not None else w.nsteps)
        assert c.status == 0
        q = dev.download(c.parity)
        frames.append(q)
        ctrls.append(c)
        t, dt = c.t, c.dt
        dev.upload(q)
    return frames, ctrls


@pytest.fixture(scope="module")
def acoustics_oracle(oracle):
    w = workloads.acoustics_radial()
    return w, oracle_frames(oracle, w)


def test_acoustics_strict_every_frame_bitwise(cuda, acoustics_oracle):
    w, (oframes, ologs) = acoustics_oracle
    frames, ctrls = device_frames(w, strict=True)
    for k, (a, b) in enumerate(zip(frames, oframes)):
        assert np.array_equal(a, b), f"frame {k}"
    for c, st in zip(ctrls, ologs):
        assert c.attempts == st["attempts"] and c.numsteps == st["numsteps"]
    assert ologs[0]["attempts"] == ologs[0]["numsteps"] + 1  # dt_initial=0.1 is rejected once


def test_acoustics_controller_run_within_1e12(cuda, acoustics_oracle):
    w, (oframes, ologs) = acoustics_oracle
    claw = workloads.make_claw(w)
    claw.run()
    assert len(claw.frames) == 11
    for k in range(11):
        assert rel_l1(claw.frames[k].q, oframes[k]) <= 1e-12, k
        if k:
            assert claw.frames[k].t == pytest.approx(0.06 * k, abs=1e-15)
    assert claw.solver.status["numsteps"] == sum(s["numsteps"] for s in ologs)


def test_host_and_device_control_agree_bitwise(cuda):
    w = workloads.acoustics_radial(60, 50)
    w.tfinal = 0.2
    res = []
    for dc in (True, False):
        claw = workloads.make_claw(w)
        claw.solver.device_control = dc
        claw.run()
        res.append([f.q for f in claw.frames] + [claw.solver.status["numsteps"]])
    for a, b in zip(res[0][:-1], res[1][:-1]):
        assert np.array_equal(a, b)
    assert res[0][-1] == res[1][-1]


@pytest.mark.parametrize("make", [
    lambda: workloads.shallow_dam_break(128, 128, nsteps=150),
    lambda: workloads.euler_quadrants(128, 96, nsteps=100),
])
def test_reduced_size_runs_match_oracle(cuda, oracle, make):
    w = make()
    oframes, ologs = oracle_frames(oracle, w)
    sframes, sctrl = device_frames(w, strict=True)
    assert np.array_equal(sframes[-1], oframes[-1])
    assert sctrl[-1].numsteps == w.nsteps == ologs[-1]["numsteps"]
    pframes, _ = device_frames(w)
    assert rel_l1(pframes[-1], oframes[-1]) <= 1e-12


def test_dam_break_full_size_properties(cuda):
    """2048^2, 1000 steps: wall boundaries conserve mass, the radial problem
    keeps its x/y mirror symmetries, and FP32 bulk stays within 1e-5 of FP64."""
    w = workloads.shallow_dam_break()
    f64, c64 = device_frames(w)
    q = f64[-1]
    assert c64[-1].numsteps == 1000
    m0, m1 = w.q0[0].sum(), q[0].sum()
    assert abs(m1 - m0) <= 1e-12 * m0
    h = q[0]
    assert np.abs(h - h[::-1, :]).max() <= 1e-10
    assert np.abs(h - h[:, ::-1]).max() <= 1e-10
    assert np.abs(h - h.T).max() <= 1e-10
    f32, c32 = device_frames(w, precision=1)
    assert c32[-1].numsteps == 1000
    assert rel_l1(f32[-1], q) <= 1e-5


def test_euler_fp32_error_bound(cuda):
    w = workloads.euler_quadrants(1024, 1024, nsteps=200)
    f64, _ = device_frames(w)
    f32, _ = device_frames(w, precision=1)
    assert rel_l1(f32[-1], f64[-1]) <= 1e-5


def test_rejections_and_fixed_dt_errors(cuda, oracle):
    w = workloads.shallow_dam_break(64, 64, nsteps=20)
    w.dt_initial = 1.0
    oframes, ologs = oracle_frames(oracle, w)
    sframes, sctrl = device_frames(w, strict=True)
    assert np.array_equal(sframes[-1], oframes[-1])
    assert sctrl[-1].attempts == ologs[-1]["attempts"] > 20
    dev = DeviceProblem(struct_of(w))
    dev.upload(w.q0)
    c = dev.evolve(0.0, 1.0, 10.0, dt_variable=False)
    assert c.status == _lib.CFL_FIXED_DT
    c = dev.evolve(0.0, 1e-5, 10.0, max_steps=7)
    assert c.status == _lib.MAX_STEPS and c.attempts == 7


def test_evolve_host_entry_point_matches(cuda):
    w = workloads.shallow_dam_break(96, 80, nsteps=40)
    frames, ctrls = device_frames(w)
    s = struct_of(w)
    L = _lib.lib()
    nb = L.gclaw_evolve_workspace_bytes(ctypes.byref(s))
    ws = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    base = (ws.data_ptr() + 255) // 256 * 256
    qin = np.asfortranarray(w.q0)
    qout = np.zeros_like(qin, order="F")
    ctrl = _lib.GclawCtrl()
    rc = L.gclaw_evolve_host(ctypes.byref(s), ctypes.c_void_p(qin.ctypes.data),
                             ctypes.c_void_p(qout.ctypes.data), 0.0, w.dt_initial, math.inf,
                             40, w.cfl_max, w.cfl_desired, 1e99, 10000, ctypes.c_void_p(base), nb,
                             8, ctypes.byref(ctrl), None)
    torch.cuda.synchronize()
    assert rc == 0 and ctrl.numsteps == 40
    assert np.array_equal(qout, frames[-1])


def test_cuda_graph_capture_of_advance(cuda):
    w = workloads.shallow_dam_break(80, 64, nsteps=30)
    frames, _ = device_frames(w)
    dev = DeviceProblem(struct_of(w))
    dev.upload(w.q0)
    dev.ctrl_init(0.0, w.dt_initial, math.inf, max_accepted=30)
    dev.advance(0)  # sets the kernel's shared-memory attribute outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            dev.advance(8, stream=s)
    # capture does not run the kernels: re-initialise, then replay
    dev.upload(w.q0)
    dev.ctrl_init(0.0, w.dt_initial, math.inf, max_accepted=30)
    torch.cuda.synchronize()
    for _ in range(5):
        g.replay()
    torch.cuda.synchronize()
    c = dev.read_ctrl()
    assert c.done and c.numsteps == 30
    assert np.array_equal(dev.download(c.parity), frames[-1])
