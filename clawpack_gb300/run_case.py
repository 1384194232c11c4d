"""Run one benchmark problem on the GPU and report its step time.

    python -m clawpack_gb300.run_case --workload shallow --mx 2048 --steps 100 \
        --precision fp64

Advances the chosen problem by --warmup then --steps device-controlled steps
(one step kernel each) and prints one JSON line with the mean step time from
CUDA events.  With --adjoint, the --warmup + --steps launches time adjoint
steps (gclaw_adjoint_step) instead, about the state after one forward step,
with a seeded random adjoint field.  Used for profiling captures and quick
size sweeps.
"""
from __future__ import annotations

import argparse
import json
import math

import torch

from . import workloads
from .device import DeviceProblem


def make_workload(name, mx, my):
    if name == "shallow":
        return workloads.shallow_dam_break(mx, my)
    if name == "euler":
        return workloads.euler_quadrants(mx, my)
    if name == "acoustics":
        return workloads.acoustics_radial(mx, my)
    raise ValueError(name)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="shallow",
                   choices=["shallow", "euler", "acoustics", "acoustics3d", "euler3d"])
    p.add_argument("--mx", type=int, default=2048)
    p.add_argument("--my", type=int, default=None)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    p.add_argument("--adjoint", action="store_true")
    p.add_argument("--fp32-kernel", default="auto", choices=["auto", "tile", "strip"])
    p.add_argument("--fp64-kernel", default="auto", choices=["auto", "tile", "strip"])
    p.add_argument("--split", action="store_true", help="dimensionally split steps")
    p.add_argument("--split-kernel", default="pencil", choices=["pencil", "tile", "march", "window"],
                   help="kernel family of 2D split steps")
    p.add_argument("--batched", type=int, default=0,
                   help="time the first N problems of the seeded shallow-water ensemble")
    a = p.parse_args(argv)
    from . import _lib

    _lib.lib().gclaw_fp32_kernel({"auto": 0, "tile": 1, "strip": 2}[a.fp32_kernel])
    _lib.lib().gclaw_fp64_kernel({"auto": 0, "tile": 1, "strip": 2}[a.fp64_kernel])
    _lib.lib().gclaw_split_kernel({"pencil": 0, "tile": 1, "march": 2, "window": 3}[a.split_kernel])
    _lib.lib().gclaw3_split_kernel({"pencil": 0, "tile": 0, "march": 1, "window": 2}[a.split_kernel])
    if a.batched:
        return run_batched(a)
    if a.workload in ("acoustics3d", "euler3d"):
        return run_3d(a)
    w = make_workload(a.workload, a.mx, a.my or a.mx)
    s = w.solver_struct(0 if a.precision == "fp64" else 1)
    dev = DeviceProblem(s, split=a.split)
    dev.upload(w.q0)
    dev.ctrl_init(0.0, w.dt_initial, math.inf, cfl_max=w.cfl_max, cfl_desired=w.cfl_desired,
                  max_steps=10 ** 9)
    if a.adjoint:
        return run_adjoint(a, w, s, dev)
    dev.advance(a.warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    dev.advance(a.steps)
    e1.record()
    c = dev.read_ctrl()
    ms = e0.elapsed_time(e1) / max(a.steps, 1)
    cells = w.mx * w.my
    print(json.dumps({"workload": w.name, "mx": w.mx, "my": w.my, "precision": a.precision,
                      "split": a.split, "steps": a.steps, "ms_per_step": ms,
                      "gcell_updates_per_s": cells / (ms * 1e-3) * 1e-9 if ms > 0 else None,
                      "accepted": c.numsteps, "status": c.status, "cfl": c.cfl}))
    return 0 if c.status == 0 else 1


def run_3d(a):
    """--warmup then --steps device-controlled 3D steps on an mx^3 cube."""
    from .device import DeviceProblem3

    w = (workloads.acoustics_3d_pulse(a.mx) if a.workload == "acoustics3d"
         else workloads.euler_3d_octants(a.mx))
    dev = DeviceProblem3(w.solver_struct(precision=0 if a.precision == "fp64" else 1),
                         split=a.split)
    dev.upload(w.q0)
    dev.ctrl_init(0.0, w.dt_initial, math.inf, cfl_max=w.cfl_max, cfl_desired=w.cfl_desired,
                  max_steps=10 ** 9)
    dev.advance(a.warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    dev.advance(a.steps)
    e1.record()
    c = dev.read_ctrl()
    ms = e0.elapsed_time(e1) / max(a.steps, 1)
    cells = w.n ** 3
    print(json.dumps({"workload": w.name, "n": w.n, "precision": a.precision, "split": a.split,
                      "steps": a.steps,
                      "ms_per_step": ms,
                      "gcell_updates_per_s": cells / (ms * 1e-3) * 1e-9 if ms > 0 else None,
                      "accepted": c.numsteps, "status": c.status, "cfl": c.cfl}))
    return 0 if c.status == 0 else 1


def run_batched(a):
    """--warmup then --steps batched launches over the first --batched
    problems of the ensemble (FP32-bulk unless --precision fp64)."""
    from . import _lib

    e = workloads.batched_ensemble(nsteps=10 ** 6)
    n = a.batched
    e.shapes, e.deltas, e.params, e.dt0 = e.shapes[:n], e.deltas[:n], e.params[:n], e.dt0[:n]
    prec = _lib.PREC_FP64 if a.precision == "fp64" else _lib.PREC_FP32_BULK
    bs = workloads.make_batch(e, precision=prec)
    bs.advance(a.warmup)
    torch.cuda.synchronize()
    c0 = bs.read_ctrls()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    bs.advance(a.steps)
    e1.record()
    torch.cuda.synchronize()
    c1 = bs.read_ctrls()
    ms = e0.elapsed_time(e1) / max(a.steps, 1)
    upd = sum(int(mx) * int(my) * int(k1 - k0) for (mx, my), k0, k1 in
              zip(e.shapes, c0["numsteps"], c1["numsteps"]))
    print(json.dumps({"workload": f"ensemble[{n}]", "cells": e.cells, "precision": a.precision,
                      "steps": a.steps, "ms_per_step": ms,
                      "gcell_updates_per_s": upd / (ms * 1e-3 * max(a.steps, 1)) * 1e-9,
                      "status_nonzero": int((c1["status"] != 0).sum())}))
    return 0 if (c1["status"] == 0).all() else 1


def run_adjoint(a, w, s, dev):
    from .adjoint import _Stepper

    dev.advance(1)
    c = dev.read_ctrl()
    q = dev.q[c.parity]
    st = _Stepper(s, q.device)
    gen = torch.Generator(device=q.device).manual_seed(5)
    lam = torch.randn(q.shape, dtype=q.dtype, device=q.device, generator=gen)
    for _ in range(a.warmup):
        lam = st.adjoint(q, lam, c.dt)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        lam = st.adjoint(q, lam, c.dt)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(a.steps, 1)
    finite = bool(torch.isfinite(lam).all())
    print(json.dumps({"workload": w.name, "mx": w.mx, "my": w.my, "precision": a.precision,
                      "adjoint_steps": a.steps, "ms_per_step": ms,
                      "gcell_updates_per_s": w.mx * w.my / (ms * 1e-3) * 1e-9 if ms > 0 else None,
                      "finite": finite}))
    return 0 if finite else 1


if __name__ == "__main__":
    raise SystemExit(main())
