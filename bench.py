#!/usr/bin/env python
"""Benchmark of the classic unsplit 2D step on GB300.

Headline workload: shallow water, Roe solver with entropy fix, 2048x2048 on
[-2.5,2.5]^2, radial dam break (h=2 for r<0.5 else 1), wall boundaries, MC
limiter, transverse_waves=2, CFL 0.9.  One bench step is one time step of
that grid; --steps K times K of them (default 1000, the full run).

Metric: Gcell-updates/s (interior cells x accepted steps / time).
  value    plain FP64 step, device-timed with CUDA events around each step
           kernel; the L2 is flushed (256 MB write) before every timed step.
  e2e      the per-step path of the reference with host buffers: every step
           moves the state from pinned host memory to the GPU, runs the step
           and moves the new state and the Courant number back
           (gclaw_step_host; pinned arrays are read and written by the step
           kernel over NVLink-C2C).  e2e_pageable: the same loop on pageable
           host arrays (numpy), staged through device buffers.
  roofline the dominant kernel (the step) against HBM bandwidth: algorithmic
           bytes 2*m*8 = 48 B per cell-update; an FP64-pipe roofline is given
           beside it because the FP64 step is bound by the FP64 units.
  cpu_baseline the CPU oracle (C restatement of the Fortran step) on the host
           cores, OpenMP over all of them, on a bounded sample of steps.
  fp32_bulk  the FP32-bulk variant (FP32 fluxes, FP64 state and CFL) on the
           same K steps, with its relative L1 error against the FP64 result.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
Under torchrun with N ranks each rank advances its own replica (the path
has no exchange step), timing is the max over ranks and value is the
aggregate over all ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("Gcell-updates/s on 1 GB300: plain FP64 vs FP32/batched at stated error; "
          "%HBM peak")
UNIT = "Gcell-updates/s"
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--mx", type=int, default=2048)
    p.add_argument("--e2e-steps", type=int, default=50)
    p.add_argument("--no-variants", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--batched-steps", type=int, default=200)
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-euler", action="store_true")
    p.add_argument("--no-3d", action="store_true")
    p.add_argument("--n3d", type=int, default=192, help="cube side of the 3D acoustics run")
    p.add_argument("--euler-steps", type=int, default=500)
    return p.parse_args()


# ------------------------------------------------------------------ plumbing
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(world, backend):
    import torch.distributed as dist

    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            d = json.load(open(path))
            hbm = d.get("hbm_gbs") or d.get("hbm_GBs")
            return float(hbm), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def profiled(kernel_tag, key):
    """A per-cell-update figure (e.g. dram_bytes_per_cell_update) from the
    committed ncu summary of a kernel, or None."""
    path = os.path.join(ROOT, "profiles", f"{kernel_tag}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------------ GPU timing
def timed_steps(dev, steps, flush, torch):
    """Time `steps` controlled step launches, one CUDA-event pair around each
    launch, flushing L2 before each.  Returns (seconds, accepted steps)."""
    stream = torch.cuda.current_stream()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    c0 = dev.read_ctrl()
    for k in range(steps):
        flush.fill_(k & 0xff)
        starts[k].record(stream)
        dev.advance(1)
        ends[k].record(stream)
    torch.cuda.synchronize()
    c1 = dev.read_ctrl()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    return ms * 1e-3, c1.numsteps - c0.numsteps, c1


def run_variant(w, precision, steps, warmup, torch, flush, world, device, split=False):
    from clawpack_gb300.device import DeviceProblem

    dev = DeviceProblem(w.solver_struct(precision), device=device, split=split)
    dev.upload(w.q0)
    dev.ctrl_init(0.0, w.dt_initial, math.inf, cfl_max=w.cfl_max, cfl_desired=w.cfl_desired,
                  max_accepted=-1, max_steps=10 ** 9)
    dev.advance(warmup)
    torch.cuda.synchronize()
    barrier(world)
    secs, accepted, c = timed_steps(dev, steps, flush, torch)
    barrier(world)
    secs = max_over_ranks(secs, world, device)
    return secs, accepted, c, dev


def e2e_host_steps(w, nsteps, torch, device, pinned=True):
    """Per-step host-buffer path through gclaw_step_host (pinned buffers, or
    pageable numpy arrays), with PyClaw's host-side dt control.  Returns
    (seconds, accepted, bytes)."""
    from clawpack_gb300 import _lib

    s = w.solver_struct(0)
    L = _lib.lib()
    nb = L.gclaw_step_workspace_bytes(ctypes.byref(s))
    ws = torch.empty(nb + 256, dtype=torch.uint8, device=device)
    base = (ws.data_ptr() + 255) // 256 * 256
    qb = w.q0.nbytes
    h = [torch.empty(qb, dtype=torch.uint8, pin_memory=pinned) for _ in range(2)]
    np.frombuffer(h[0].numpy(), dtype=np.float64)[:] = np.asfortranarray(w.q0).ravel(order="F")
    cfl = ctypes.c_double()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    dt = w.dt_initial
    src, accepted = 0, 0
    # one untimed call to load the module and set kernel attributes
    rc = L.gclaw_step_host(ctypes.byref(s), ctypes.c_void_p(h[0].data_ptr()),
                           ctypes.c_void_p(h[1].data_ptr()), dt, ctypes.c_void_p(base), nb,
                           ctypes.byref(cfl), sp)
    _lib.check(rc, "gclaw_step_host")
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(nsteps):
        rc = L.gclaw_step_host(ctypes.byref(s), ctypes.c_void_p(h[src].data_ptr()),
                               ctypes.c_void_p(h[1 - src].data_ptr()), dt,
                               ctypes.c_void_p(base), nb, ctypes.byref(cfl), sp)
        _lib.check(rc, "gclaw_step_host")
        if cfl.value <= w.cfl_max:
            accepted += 1
            src ^= 1
        dt = min(1e99, dt * w.cfl_desired / cfl.value)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return max(e0.elapsed_time(e1) * 1e-3, wall), accepted, qb


def bench_batched(args, torch, world, device):
    """4096 independent shallow-water problems (32^2..512^2, 193 M cells),
    FP32 bulk, each with its own dt/CFL, `batched_steps` steps from one CUDA
    graph of batched launches (working set 9.3 GB, far above L2)."""
    from clawpack_gb300 import _lib, workloads

    n = args.batched_steps
    e = workloads.batched_ensemble(nsteps=n)
    bs = workloads.make_batch(e, device=device)
    bs.advance(3)  # warm-up launches
    torch.cuda.synchronize()
    graph = bs.capture(n)
    # restart from the initial state for the timed replay
    host = bs.pinned_host_buffer()
    for p in range(len(e.shapes)):
        bs.pack(host, p, e.q0(p))
    bs.upload(host)
    bs.ctrl_init(e.dt0, cfl_max=e.cfl_max, cfl_desired=e.cfl_desired, max_accepted=n,
                 max_steps=10 * n)
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    graph.replay()
    e1.record()
    torch.cuda.synchronize()
    secs = max_over_ranks(e0.elapsed_time(e1) * 1e-3, world, device)
    ctrl = bs.read_ctrls()
    updates = int(sum(int(a) * int(b) * int(k) for (a, b), k in zip(e.shapes, ctrl["numsteps"])))
    del bs, graph, host
    torch.cuda.empty_cache()
    # FP32 error against FP64 on the first 128 problems
    sub = workloads.batched_ensemble(nsteps=n)
    sub.shapes, sub.deltas, sub.params, sub.dt0 = (sub.shapes[:128], sub.deltas[:128],
                                                   sub.params[:128], sub.dt0[:128])
    res = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_FP32_BULK):
        b = workloads.make_batch(sub, precision=prec, device=device)
        b.advance(n + 10)
        res[prec] = b.download()
    errs = [float(np.abs(a - r).sum() / np.abs(r).sum())
            for a, r in zip(res[_lib.PREC_FP32_BULK], res[_lib.PREC_FP64])]
    return {"value": round(world * updates / secs * 1e-9, 4), "unit": UNIT,
            "workload": f"{len(e.shapes)} shallow-water problems, sides log-uniform 32..512 "
                        f"({e.cells} cells), FP32 bulk, per-problem dt/CFL, {n} steps",
            "ms_per_step": round(secs / n * 1e3, 3), "accepted_cell_updates": updates,
            "all_problems_done": bool(np.all(ctrl["done"] == 1)),
            "status_nonzero": int(np.sum(ctrl["status"] != 0)),
            "launches": n, "cuda_graph": True,
            "rel_l1_vs_fp64_max_over_128_problems": max(errs)}


def bench_euler(args, torch, world, device):
    """Four-quadrant Euler problem, 4096^2, superbee, CFL 0.8: FP32-bulk and
    FP64 step rates over `euler_steps` steps (537 MB per state buffer, above
    L2, so no flush) and the FP32-bulk error against the FP64 run."""
    from clawpack_gb300 import workloads
    from clawpack_gb300.device import DeviceProblem

    n = args.euler_steps
    small = workloads.euler_quadrants(128, 128, nsteps=3)
    w = workloads.euler_quadrants(nsteps=n)
    res, finals = {}, {}
    for name, prec in (("fp32_bulk", 1), ("fp64", 0)):
        for prob, steps in ((small, 3), (w, n)):  # the small run loads the kernel
            dev = DeviceProblem(prob.solver_struct(prec), device=device)
            dev.upload(prob.q0)
            dev.ctrl_init(0.0, prob.dt_initial, math.inf, cfl_max=prob.cfl_max,
                          cfl_desired=prob.cfl_desired, max_accepted=steps, max_steps=10 * steps)
            torch.cuda.synchronize()
            barrier(world)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dev.advance(steps)
            e1.record()
            torch.cuda.synchronize()
        secs = max_over_ranks(e0.elapsed_time(e1) * 1e-3, world, device)
        c = dev.read_ctrl()
        finals[name] = dev.q[c.parity].clone()
        res[name] = {"value": round(world * w.mx * w.my * c.numsteps / secs * 1e-9, 4),
                     "ms_per_step": round(secs / n * 1e3, 4), "accepted_steps": int(c.numsteps),
                     "attempts": int(c.attempts)}
        del dev
    a, b = finals["fp32_bulk"], finals["fp64"]
    return {"workload": f"euler_quadrants {w.mx}x{w.my} 4-wave Roe + efix, superbee, extrap BCs, "
                        f"CFL 0.8, {n} steps (seed {w.meta['seed']})",
            "unit": UNIT, **res,
            "fp32_rel_l1_vs_fp64": float((a - b).abs().sum() / b.abs().sum()),
            "launches": 2 * n}  # one step kernel per attempt in each timed run


def bench_3d(args, torch, world, device):
    """3D steps (classic3, acoustics_3D, MC): a pressure pulse between walls
    on an n^3 cube, unsplit with transverse_waves 22 and dimensionally split,
    FP64 and FP32-bulk, 40 device-controlled steps each (1.7 GB of state and
    workspace per 192^3, above L2); euler_3D on the octant problem; and the
    CPU oracle on a 48^3 cube for reference."""
    from clawpack_gb300 import workloads
    from clawpack_gb300.device import DeviceProblem3

    def timed(make, n, k, prec, split=False):
        # a 32^3 warm-up run of the same kernels, then k device-controlled
        # steps on the n^3 problem
        for prob, kk in ((make(32), 3), (make(n), k)):
            dev = DeviceProblem3(prob.solver_struct(precision=prec), device=device, split=split)
            dev.upload(prob.q0)
            dev.ctrl_init(0.0, prob.dt_initial, math.inf, cfl_max=prob.cfl_max,
                          cfl_desired=prob.cfl_desired, max_accepted=kk, max_steps=10 * kk)
            torch.cuda.synchronize()
            barrier(world)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dev.advance(kk)
            e1.record()
            torch.cuda.synchronize()
            secs = max_over_ranks(e0.elapsed_time(e1) * 1e-3, world, device)
            c = dev.read_ctrl()
        # kernels per step attempt in the timed n^3 run: three sweeps of one
        # kernel each (split sweeps, and the fused FP32-bulk sweep), or of
        # the three staged kernels (FP64 with transverse terms)
        per_step = 3 if split or prec == 1 else 9
        res = {"value": round(world * n ** 3 * c.numsteps / secs * 1e-9, 4),
               "ms_per_step": round(secs / k * 1e3, 3),
               "accepted_steps": int(c.numsteps), "status": int(c.status),
               "launches": per_step * k}
        return res, dev.q[c.parity].clone()

    n, steps = args.n3d, 40
    out = {"workload": f"acoustics_3d_pulse {n}^3, wall BCs, MC, transverse_waves 22 "
                       f"(corner transport), CFL 0.9, {steps} steps",
           "unit": UNIT}
    finals = {}
    for name, prec in (("fp64", 0), ("fp32_bulk", 1)):
        out[name], finals[name] = timed(workloads.acoustics_3d_pulse, n, steps, prec)
    a, b = finals["fp32_bulk"], finals["fp64"]
    out["fp32_rel_l1_vs_fp64"] = float((a - b).abs().sum() / b.abs().sum())
    # ClawSolver3D's default: dimensionally split sweeps, same problem
    out["split"] = {"workload": f"acoustics_3d_pulse {n}^3, dimensionally split, MC, "
                                f"{steps} steps"}
    for name, prec in (("fp64", 0), ("fp32_bulk", 1)):
        out["split"][name], _ = timed(workloads.acoustics_3d_pulse, n, steps, prec, split=True)
    # 3D Euler (euler_3D, Roe, three wave families) on the seeded octant
    # problem, 128^3, extrapolation boundaries, MC limiter, CFL 0.8
    ne, esteps = 128, 20
    eu = {"workload": f"euler_3d_octants {ne}^3 (seed {workloads.EULER3D_SEED}), extrap BCs, "
                      f"MC, transverse_waves 22, CFL 0.8, {esteps} steps"}
    for name, prec in (("fp64", 0), ("fp32_bulk", 1)):
        eu[name], _ = timed(workloads.euler_3d_octants, ne, esteps, prec)
    out["euler_3d"] = eu
    # launches inside the timed regions of this leg
    out["launches"] = sum(leg[name]["launches"] for leg in (out, out["split"], eu)
                          for name in ("fp64", "fp32_bulk"))
    if int(os.environ.get("RANK", "0")) == 0:
        from oracle import ref
        small = workloads.acoustics_3d_pulse(48)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref.step3(1, small.problem_data, small.q0, *small.delta, small.dt_initial,
                  small.bc_lower, small.bc_upper, 2, 22, [4, 4], nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(48 ** 3 / dt * 1e-9, 5), "unit": UNIT,
                               "cores": threads, "kind": "port",
                               "sample": "one 48^3 step of the same problem, CPU oracle"}
    return out


def bench_adjoint(torch, world, device):
    """Gradient of the gauge least-squares loss with respect to the initial
    surface: 1024^2 shallow water, 500 steps, checkpoints every 23 steps,
    64 gauges; forward + checkpointed backward through the hand-written
    adjoint kernel, FP64 and FP32-bulk."""
    from clawpack_gb300 import _lib, adjoint, workloads

    p = workloads.adjoint_problem()
    s64 = p.solver_struct(_lib.PREC_FP64)
    dts = adjoint.record_dts(torch.from_numpy(p.q0()).to(device), s64, p.nsteps, p.dt0)
    gauges = torch.as_tensor(p.gauges, device=device)
    target = adjoint.gauge_series(torch.from_numpy(p.q0(p.h_true)).to(device), s64, dts, gauges)
    warm = workloads.adjoint_problem(64, nsteps=8, checkpoint_every=3)
    res, grads = {}, {}
    for name, prec in (("fp64", _lib.PREC_FP64), ("fp32_bulk", _lib.PREC_FP32_BULK)):
        for prob, d, tg in ((warm, dts[:8], None), (p, dts, target)):
            h0 = torch.from_numpy(prob.h0).to(device).requires_grad_(True)
            q = torch.stack([h0, torch.zeros_like(h0), torch.zeros_like(h0)])
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            torch.cuda.synchronize()
            barrier(world)
            ev[0].record()
            series = adjoint.evolve_gauges(q, prob.solver_struct(prec), d,
                                           torch.as_tensor(prob.gauges, device=device),
                                           prob.checkpoint_every)
            ev[1].record()
            loss = ((series - (series.detach() * 0 if tg is None else tg)) ** 2).sum()
            loss.backward()
            ev[2].record()
            torch.cuda.synchronize()
        fwd = max_over_ranks(ev[0].elapsed_time(ev[1]) * 1e-3, world, device)
        bwd = max_over_ranks(ev[1].elapsed_time(ev[2]) * 1e-3, world, device)
        grads[name] = h0.grad.double().cpu().numpy()
        cells = p.mx * p.my
        n = len(dts)
        res[name] = {"forward_s": round(fwd, 4), "backward_s": round(bwd, 4),
                     "gradient_s": round(fwd + bwd, 4),
                     "forward_gcell_updates_per_s": round(world * cells * n / fwd * 1e-9, 4),
                     "backward_gcell_updates_per_s": round(world * cells * n / bwd * 1e-9, 4),
                     "loss": float(loss.detach())}
    a, b = grads["fp64"], grads["fp32_bulk"]
    nseg = -(-len(dts) // p.checkpoint_every)
    return {"workload": f"shallow water {p.mx}x{p.my}, {len(dts)} steps, 64 gauges, "
                        f"checkpoints every {p.checkpoint_every} steps, MC, wall BCs",
            "unit": "s per gradient", **res,
            "fp32_vs_fp64_grad_rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(a)),
            "launches_per_gradient": 2 * len(dts) + (len(dts) - nseg),
            "launches": 2 * (2 * len(dts) + (len(dts) - nseg))}


def cpu_model():
    """The host CPU's model name as lscpu reports it (the machine type if
    lscpu is missing)."""
    import platform

    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":", 1)[0].strip() == "Model name":
                return f"{line.split(':', 1)[1].strip()} ({platform.machine()})"
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.machine()


def cpu_baseline(w, target_s=15.0):
    """The CPU oracle on the host cores (OpenMP, all threads) over a bounded
    number of full-grid steps."""
    from oracle import ref

    threads = os.cpu_count() or 1
    ref.lib()
    q = w.q0
    dt = w.dt_initial

    def one(q, dt):
        return ref.step(w.rp_id, w.pd_array(), q, w.dx, w.dy, dt, w.bc_lower, w.bc_upper,
                        w.order, w.transverse_waves, w.mthlim(), nthreads=threads)

    t0 = time.perf_counter()
    q, cfl, _ = one(q, dt)
    first = time.perf_counter() - t0
    n = int(max(1, min(1000, target_s / max(first, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(n):
        dt = dt * w.cfl_desired / cfl
        q, cfl, _ = one(q, dt)
    secs = time.perf_counter() - t0
    cells = w.mx * w.my
    # one thread, as the reference's serial step runs
    n1, t1 = 0, time.perf_counter()
    while n1 == 0 or (time.perf_counter() - t1 < target_s / 2 and n1 < 50):
        q1, cfl1, _ = ref.step(w.rp_id, w.pd_array(), w.q0, w.dx, w.dy, w.dt_initial,
                               w.bc_lower, w.bc_upper, w.order, w.transverse_waves, w.mthlim(),
                               nthreads=1)
        n1 += 1
    secs1 = time.perf_counter() - t1
    return {"value": cells * n / secs * 1e-9, "unit": UNIT, "cores": threads, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": f"{n} full {w.mx}x{w.my} steps of the same problem on {threads} threads "
                      f"(OpenMP over slices), {secs:.1f} s",
            "one_thread": {"value": cells * n1 / secs1 * 1e-9, "cores": 1,
                           "sample": f"{n1} full {w.mx}x{w.my} steps on one thread, {secs1:.1f} s"}}


# ------------------------------------------------------------------ arms
def run_ours(args):
    import torch

    world, rank, local = dist_env()
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    init_dist(world, "nccl")
    from clawpack_gb300 import workloads

    w = workloads.shallow_dam_break(args.mx, args.mx, nsteps=args.warmup + args.steps)
    m = w.num_eqn
    cells = w.mx * w.my
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    peak, peak_kind = measured_peaks()

    clocks = ClockSampler(local).start()
    secs, accepted, c64, dev64 = run_variant(w, 0, args.steps, args.warmup, torch, flush, world,
                                             device)
    clk = clocks.stop()
    value = world * cells * accepted / secs * 1e-9
    t_kernel = secs / args.steps
    alg_bytes = 2 * m * 8 * cells
    achieved = alg_bytes / t_kernel * 1e-9
    traffic_per_cell = profiled("step_fp64_shallow", "dram_bytes_per_cell_update")
    fp64_inst = profiled("step_fp64_shallow", "fp64_inst_per_cell_update")
    sm_mhz = clk.get("sm_mhz") or 2070.0
    fp64_peak = 152 * 2 * sm_mhz * 1e6  # FP64 thread-instructions per second (2/clk/SM)
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(secs / args.steps * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"shallow_dam_break {w.mx}x{w.my} Roe+efix, wall BCs, MC, "
                               "transverse_waves=2, CFL 0.9, FP64",
                   "mx": w.mx, "my": w.my, "accepted_steps": accepted,
                   "l2": "flushed before every timed step (256 MB write, untimed)",
                   "parallelism": f"replicas x{world}",
                   "seeds": {"euler": workloads.EULER_SEED, "batched": workloads.BATCH_SEED,
                             "adjoint": workloads.ADJOINT_SEED}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": f"{peak_kind} HBM copy bandwidth",
                     "traffic": (None if traffic_per_cell is None
                                 else round(traffic_per_cell * cells)),
                     "alg_bytes_per_launch": alg_bytes,
                     "note": "the FP64 step is bound by the FP64 pipe, not HBM"},
        "roofline_fp64_pipe": (None if fp64_inst is None else {
            "bound": "fp64 pipe", "inst_per_cell_update": fp64_inst,
            "peak_inst_per_s": fp64_peak, "bound_gcell_updates_per_s": fp64_peak / fp64_inst * 1e-9,
            "frac": round(value / world / (fp64_peak / fp64_inst * 1e-9), 4),
            "source": "FP64 instruction count per cell-update from profiles/step_fp64_shallow.md"}),
        "clocks": clk,
        "gpu_launches": args.steps,
    }
    if not args.no_variants:
        s32, acc32, c32, dev32 = run_variant(w, 1, args.steps, args.warmup, torch, flush, world,
                                             device)
        v32 = world * cells * acc32 / s32 * 1e-9
        q64 = dev64.q[c64.parity]
        q32 = dev32.q[c32.parity]
        err = float((q32 - q64).abs().sum() / q64.abs().sum())
        a32 = alg_bytes / (s32 / args.steps) * 1e-9
        t32 = profiled("strip_fp32_shallow", "dram_bytes_per_cell_update")
        out["fp32_bulk"] = {"value": round(v32, 4), "unit": UNIT, "dtype": "f32 fluxes, f64 q",
                            "rel_l1_vs_fp64": err, "speedup_vs_fp64": round(v32 / value, 3),
                            "ms_per_step": round(s32 / args.steps * 1e3, 4),
                            "roofline": {"bound": "hbm", "achieved": round(a32, 1),
                                         "peak": peak, "unit": "GB/s",
                                         "frac": round(a32 / peak, 4),
                                         "traffic": None if t32 is None else round(t32 * cells)}}
        out["gpu_launches"] += args.steps
        del dev32
        # ClawSolver2D's default: dimensionally split steps (x-sweep, boundary
        # conditions, y-sweep), one pencil kernel per sweep; the state is read
        # and written once per sweep: 2 x 2 x 24 B per cell-update
        sp = {"workload": f"{w.name} {w.mx}x{w.my}, dimensionally split (ClawSolver2D "
                          f"default), same step sequence rules",
              "unit": UNIT, "alg_bytes_per_cell_update": 96}
        for name, prec in (("fp64", 0), ("fp32_bulk", 1)):
            ss, accs, cs, devs = run_variant(w, prec, args.steps, args.warmup, torch, flush, world,
                                             device, split=True)
            ach = 96 * cells / (ss / args.steps) * 1e-9
            sp[name] = {"value": round(world * cells * accs / ss * 1e-9, 4),
                        "ms_per_step": round(ss / args.steps * 1e3, 4),
                        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak,
                                     "unit": "GB/s", "frac": round(ach / peak, 4)}}
            del devs
        out["split"] = sp
        out["gpu_launches"] += 4 * args.steps
    if not args.no_batched:
        out["batched"] = bench_batched(args, torch, world, device)
        out["gpu_launches"] += out["batched"]["launches"]
    if not args.no_euler:
        out["euler"] = bench_euler(args, torch, world, device)
        out["gpu_launches"] += out["euler"]["launches"]
    if not args.no_3d:
        out["acoustics_3d"] = bench_3d(args, torch, world, device)
        out["gpu_launches"] += out["acoustics_3d"]["launches"]
    if not args.no_adjoint:
        out["adjoint"] = bench_adjoint(torch, world, device)
        out["gpu_launches"] += out["adjoint"]["launches"]
    # end to end through the C ABI with host buffers, every step
    e2e_s, e2e_acc, qb = e2e_host_steps(w, args.e2e_steps, torch, device)
    e2e_s = max_over_ranks(e2e_s, world, device)
    out["e2e"] = {"value": round(world * cells * e2e_acc / e2e_s * 1e-9, 4), "unit": UNIT,
                  "h2d_bytes_per_step": qb, "d2h_bytes_per_step": qb + 8 + 4,
                  "steps": args.e2e_steps,
                  "path": "gclaw_step_host every step: pinned host q read by the fused BC + "
                          "step kernel over NVLink-C2C, new q written to pinned host memory, "
                          "CFL -> host, host dt control"}
    p_s, p_acc, _ = e2e_host_steps(w, args.e2e_steps, torch, device, pinned=False)
    p_s = max_over_ranks(p_s, world, device)
    out["e2e_pageable"] = {"value": round(world * cells * p_acc / p_s * 1e-9, 4), "unit": UNIT,
                           "path": "gclaw_step_host every step on pageable host arrays: "
                                   "copies through device buffers, four bands overlapping "
                                   "the copies"}
    if rank == 0 and world == 1 and not args.no_cpu:
        cw = w
        out["cpu_baseline"] = cpu_baseline(cw)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_reference(args):
    """The reference arm: the CPU oracle (the reference Fortran step cannot
    be built here; its restatement is timed instead) on the host cores, each
    step one time step of a bounded 2048 x 128 band of the same problem."""
    world, rank, _ = dist_env()
    if world > 1 and rank != 0:
        return
    from clawpack_gb300 import workloads
    from oracle import ref

    threads = os.cpu_count() or 1
    band = 128
    w = workloads.shallow_dam_break(args.mx, args.mx)
    lo = args.mx // 2 - band // 2
    q = np.asfortranarray(w.q0[:, :, lo:lo + band])
    ref.lib()
    dt = w.dt_initial
    cfl = w.cfl_desired

    def one(q, dt):
        return ref.step(w.rp_id, w.pd_array(), q, w.dx, w.dy, dt, w.bc_lower, w.bc_upper,
                        w.order, w.transverse_waves, w.mthlim(), nthreads=threads)

    for _ in range(args.warmup):
        q, cfl, _ = one(q, dt)
        dt = dt * w.cfl_desired / cfl
    t0 = time.perf_counter()
    for _ in range(args.steps):
        q, cfl, _ = one(q, dt)
        dt = dt * w.cfl_desired / cfl
    secs = time.perf_counter() - t0
    cells = args.mx * band
    v = cells * args.steps / secs * 1e-9
    sample = (f"each step: one time step of a {args.mx}x{band} band through the dam "
              f"(same dx, dt rule, BCs), CPU oracle on {threads} threads")
    out = {"impl": "reference", "metric": METRIC, "value": round(v, 5), "unit": UNIT,
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(secs / args.steps * 1e3, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"shallow_dam_break {args.mx}x{args.mx} band sample",
                      "band_rows": band},
           "cpu_baseline": {"value": round(v, 5), "unit": UNIT, "cores": threads,
                            "kind": "port", "cpu_model": cpu_model(), "sample": sample},
           "e2e": {"value": round(v, 5), "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
