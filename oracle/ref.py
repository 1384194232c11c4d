"""ctypes front end of the CPU oracle, plus PyClaw's time-step control loop.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``; the product (clawpack_gb300) never
imports it.  PARITY UNPINNED -- see the header of ``classic2_ref.c``.

``evolve`` restates upstream pyclaw/src/pyclaw/solver.py ``evolve_to_time``
(absent from the mounted reference tree): clip dt to land on tend, take a
step, reject it when the Courant number exceeds cfl_max, then
dt = min(dt_max, dt * cfl_desired / cfl).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libclassic2_ref.so")

RP_ACOUSTICS, RP_SHALLOW, RP_EULER, RP_VC_ACOUSTICS, RP_SHALLOW_FWAVE = 1, 2, 3, 4, 5
SHAPES = {RP_ACOUSTICS: (3, 2), RP_SHALLOW: (3, 3), RP_EULER: (4, 4), RP_VC_ACOUSTICS: (3, 2),
          RP_SHALLOW_FWAVE: (3, 3)}

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.gclaw_ref_step.argtypes = [ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, dp, dp,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int, ip, ip, ip, dp, ctypes.c_int]
        L.gclaw_ref_step2.argtypes = [ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, ctypes.c_int, ip, dp, ctypes.c_int]
        L.gclaw_ref_step_split.argtypes = [ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, dp, dp,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int, ip, ip, ip, dp, ctypes.c_int]
        L.gclaw_ref_step2ds.argtypes = [ctypes.c_int, dp, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, ip, ctypes.c_int, dp,
                                        ctypes.c_int]
        L.gclaw_ref_fill_ghosts.argtypes = [ctypes.c_int] * 4 + [ip, ip, dp, dp]
        L.gclaw_ref_fill_aux_ghosts.argtypes = [ctypes.c_int] * 4 + [ip, ip, dp, dp]
        L.gclaw_ref_step_aux.argtypes = [ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, dp, dp,
                                         ctypes.c_int, dp, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_int, ip, ip, ip,
                                         ip, ip, dp, ctypes.c_int, ctypes.c_int]
        L.gclaw_ref_step2_aux.argtypes = [ctypes.c_int, dp, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, dp, dp, ctypes.c_int, dp, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_int, ip, dp, ctypes.c_int, ctypes.c_int]
        L.gclaw_ref_rpn2_aux.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, dp, dp, dp, dp, dp,
                                         dp, dp]
        L.gclaw_ref_rpt2_aux.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, dp, dp, dp, dp, dp]
        L.gclaw_ref_rpn2.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, dp, dp, dp, dp, dp]
        L.gclaw_ref_rpt2.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, dp, dp, dp, dp]
        L.gclaw_ref_philim.argtypes = [ctypes.c_int, ctypes.c_double]
        L.gclaw_ref_philim.restype = ctypes.c_double
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _pd(pd):
    out = np.zeros(8)
    out[:len(pd)] = pd
    return out


def to_fortran_flat(q):
    """(m, mx, my) array -> contiguous buffer in Fortran order."""
    return np.asfortranarray(q)


def fill_ghosts(q, bc_lower, bc_upper):
    m, mx, my = q.shape
    qf = np.asfortranarray(q, dtype=np.float64)
    qbc = np.zeros((m, mx + 4, my + 4), order="F")
    rc = lib().gclaw_ref_fill_ghosts(m, mx, my, 2, _ip(np.array(bc_lower, np.int32)),
                                     _ip(np.array(bc_upper, np.int32)), _dp(qf), _dp(qbc))
    if rc:
        raise ValueError(f"gclaw_ref_fill_ghosts failed: {rc}")
    return qbc


def step2(rp, pd, qbc, dx, dy, dt, order=2, tw=2, mthlim=(4, 4, 4, 4), nthreads=1):
    """The unsplit step on a ghost-filled qbc; returns (qnew_bc, cfl)."""
    m, nx, ny = qbc.shape
    qold = np.asfortranarray(qbc, dtype=np.float64)
    qnew = np.zeros_like(qold, order="F")
    cfl = np.zeros(1)
    lim = np.zeros(4, np.int32)
    lim[:len(mthlim)] = mthlim
    rc = lib().gclaw_ref_step2(rp, _dp(_pd(pd)), 2, nx - 4, ny - 4, _dp(qold), _dp(qnew), dx, dy,
                               dt, order, tw, _ip(lim), _dp(cfl), nthreads)
    if rc < 0:
        raise ValueError(f"gclaw_ref_step2 failed: {rc}")
    return qnew, float(cfl[0])


def step(rp, pd, q, dx, dy, dt, bc_lower, bc_upper, order=2, tw=2, mthlim=(4, 4, 4, 4),
         nthreads=1):
    """Ghost fill + step on an interior (m, mx, my) array; returns (qnew, cfl, rc)."""
    m, mx, my = q.shape
    qf = np.asfortranarray(q, dtype=np.float64)
    qout = np.zeros_like(qf, order="F")
    cfl = np.zeros(1)
    lim = np.zeros(4, np.int32)
    lim[:len(mthlim)] = mthlim
    rc = lib().gclaw_ref_step(rp, _dp(_pd(pd)), mx, my, _dp(qf), _dp(qout), dx, dy, dt, order,
                              tw, _ip(lim), _ip(np.array(bc_lower, np.int32)),
                              _ip(np.array(bc_upper, np.int32)), _dp(cfl), nthreads)
    if rc < 0:
        raise ValueError(f"gclaw_ref_step failed: {rc}")
    return qout, float(cfl[0]), rc


def step_aux(rp, pd, q, aux, dx, dy, dt, bc_lower, bc_upper, aux_bc_lower, aux_bc_upper,
             order=2, tw=2, mthlim=(4, 4, 4, 4), nthreads=1, mcapa=0):
    """Ghost fill of q and aux + step with an aux array (maux, mx, my); mcapa
    is the 1-based capacity field of aux (0: none).  Returns (qnew, cfl,
    rc)."""
    m, mx, my = q.shape
    qf = np.asfortranarray(q, dtype=np.float64)
    af = np.asfortranarray(aux, dtype=np.float64)
    qout = np.zeros_like(qf, order="F")
    cfl = np.zeros(1)
    lim = np.zeros(4, np.int32)
    lim[:len(mthlim)] = mthlim
    i32 = lambda v: _ip(np.array(v, np.int32))  # noqa: E731
    rc = lib().gclaw_ref_step_aux(rp, _dp(_pd(pd)), mx, my, _dp(qf), _dp(qout), af.shape[0],
                                  _dp(af), dx, dy, dt, order, tw, _ip(lim), i32(bc_lower),
                                  i32(bc_upper), i32(aux_bc_lower), i32(aux_bc_upper), _dp(cfl),
                                  nthreads, mcapa)
    if rc < 0:
        raise ValueError(f"gclaw_ref_step_aux failed: {rc}")
    return qout, float(cfl[0]), rc


def fill_aux_ghosts(aux, bc_lower, bc_upper):
    maux, mx, my = aux.shape
    af = np.asfortranarray(aux, dtype=np.float64)
    abc = np.zeros((maux, mx + 4, my + 4), order="F")
    rc = lib().gclaw_ref_fill_aux_ghosts(maux, mx, my, 2, _ip(np.array(bc_lower, np.int32)),
                                         _ip(np.array(bc_upper, np.int32)), _dp(af), _dp(abc))
    if rc:
        raise ValueError(f"gclaw_ref_fill_aux_ghosts failed: {rc}")
    return abc


def rpn2_aux(rp, pd, ixy, ql, qr, al, ar):
    m, mw = SHAPES[rp]
    wave, s, amdq, apdq = np.zeros(mw * m), np.zeros(mw), np.zeros(m), np.zeros(m)
    f = lambda a: _dp(np.ascontiguousarray(a, float))  # noqa: E731
    rc = lib().gclaw_ref_rpn2_aux(rp, _dp(_pd(pd)), ixy, f(ql), f(qr), f(al), f(ar), _dp(wave),
                                  _dp(s), _dp(amdq), _dp(apdq))
    return wave.reshape(mw, m), s, amdq, apdq, rc


def rpt2_aux(rp, pd, ixy, am, a0, ap, asdq):
    m = SHAPES[rp][0]
    bm, bp = np.zeros(m), np.zeros(m)
    f = lambda a: _dp(np.ascontiguousarray(a, float))  # noqa: E731
    lib().gclaw_ref_rpt2_aux(rp, _dp(_pd(pd)), ixy, f(am), f(a0), f(ap), f(asdq), _dp(bm),
                             _dp(bp))
    return bm, bp


def step_split(rp, pd, q, dx, dy, dt, bc_lower, bc_upper, order=2, mthlim=(4, 4, 4, 4),
               nthreads=1):
    """PyClaw's dimensionally split step (x-sweep, boundary conditions, y-sweep)
    on an interior (m, mx, my) array; returns (qnew, cfl, rc)."""
    m, mx, my = q.shape
    qf = np.asfortranarray(q, dtype=np.float64)
    qout = np.zeros_like(qf, order="F")
    cfl = np.zeros(1)
    lim = np.zeros(4, np.int32)
    lim[:len(mthlim)] = mthlim
    rc = lib().gclaw_ref_step_split(rp, _dp(_pd(pd)), mx, my, _dp(qf), _dp(qout), dx, dy, dt,
                                    order, _ip(lim), _ip(np.array(bc_lower, np.int32)),
                                    _ip(np.array(bc_upper, np.int32)), _dp(cfl), nthreads)
    if rc < 0:
        raise ValueError(f"gclaw_ref_step_split failed: {rc}")
    return qout, float(cfl[0]), rc


def rpn2(rp, pd, ixy, ql, qr):
    m, mw = SHAPES[rp]
    wave = np.zeros(mw * m)
    s = np.zeros(mw)
    amdq = np.zeros(m)
    apdq = np.zeros(m)
    rc = lib().gclaw_ref_rpn2(rp, _dp(_pd(pd)), ixy, _dp(np.ascontiguousarray(ql, float)),
                              _dp(np.ascontiguousarray(qr, float)), _dp(wave), _dp(s), _dp(amdq),
                              _dp(apdq))
    return wave.reshape(mw, m), s, amdq, apdq, rc


def rpt2(rp, pd, ixy, ql, qr, asdq):
    m, _ = SHAPES[rp]
    bm = np.zeros(m)
    bp = np.zeros(m)
    lib().gclaw_ref_rpt2(rp, _dp(_pd(pd)), ixy, _dp(np.ascontiguousarray(ql, float)),
                         _dp(np.ascontiguousarray(qr, float)),
                         _dp(np.ascontiguousarray(asdq, float)), _dp(bm), _dp(bp))
    return bm, bp


def philim(lim_id, r):
    return lib().gclaw_ref_philim(lim_id, float(r))


class Status(dict):
    pass


def evolve(step_fn, q, t, tend, dt, *, cfl_max=1.0, cfl_desired=0.9, dt_max=1e99,
           max_steps=10000, max_accepted=None):
    """PyClaw's evolve_to_time with variable dt.  step_fn(q, dt) -> (qnew, cfl).

    If ``max_accepted`` is given, the loop also stops after that many accepted
    steps (used for fixed-step-count workloads with tend = inf).
    Returns (q, t, dt, status) where status holds numsteps, attempts,
    cflmax, dtmin, dtmax and the list of (dt, cfl, accepted) per attempt.
    """
    tstart = t
    st = Status(numsteps=0, attempts=0, cflmax=0.0, dtmin=dt, dtmax=dt, log=[])
    for _ in range(max_steps):
        if max_accepted is None:
            if t + dt > tend and tstart < tend:
                dt = tend - t
            if tend - t - dt < 1.0e-14 * t:
                dt = tend - t
        qnew, cfl = step_fn(q, dt)
        st["attempts"] += 1
        if np.isnan(cfl):
            raise FloatingPointError("CFL is NaN")
        accepted = cfl <= cfl_max
        st["log"].append((dt, cfl, accepted))
        if accepted:
            st["cflmax"] = max(cfl, st["cflmax"])
            t += dt
            q = qnew
            st["numsteps"] += 1
        if t >= tend:
            break
        if max_accepted is not None and st["numsteps"] >= max_accepted:
            break
        if cfl > 0.0:
            dt = min(dt_max, dt * cfl_desired / cfl)
            st["dtmin"] = min(dt, st["dtmin"])
            st["dtmax"] = max(dt, st["dtmax"])
        else:
            dt = dt_max
    else:
        if max_accepted is None and t < tend:
            raise RuntimeError("Maximum number of timesteps have been taken")
    return q, t, dt, st


# ---------------------------------------------------------------------------
# 3D (classic3_ref.c): the unsplit 3D step.  q arrays are (m, mx, my, mz).
# ---------------------------------------------------------------------------
LIB3 = os.path.join(HERE, "libclassic3_ref.so")
RP3_ACOUSTICS, RP3_EULER, RP3_ADVECTION = 1, 2, 100
SHAPES3 = {RP3_ACOUSTICS: (4, 2), RP3_EULER: (5, 3), RP3_ADVECTION: (1, 1)}
_lib3 = None


def lib3():
    global _lib3
    if _lib3 is None:
        if not os.path.exists(LIB3):
            build()
        L = ctypes.CDLL(LIB3)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        i, d = ctypes.c_int, ctypes.c_double
        L.gclaw3_ref_fill_ghosts.argtypes = [i, i, i, i, i, ip, ip, dp, dp]
        L.gclaw3_ref_step3.argtypes = [i, dp, i, i, i, dp, dp, d, d, d, d, i, i, ip, dp, i]
        L.gclaw3_ref_step.argtypes = [i, dp, i, i, i, dp, dp, d, d, d, d, i, i, ip, ip, ip, dp, i]
        L.gclaw3_ref_rpn3.argtypes = [i, dp, i, dp, dp, dp, dp, dp, dp]
        L.gclaw3_ref_step_split.argtypes = [i, dp, i, i, i, dp, dp, d, d, d, d, i, ip, ip, ip,
                                            dp, i]
        _lib3 = L
    return _lib3


def fill_ghosts3(q, bc_lower, bc_upper):
    m, mx, my, mz = q.shape
    qf = np.asfortranarray(q, dtype=np.float64)
    qbc = np.zeros((m, mx + 4, my + 4, mz + 4), order="F")
    rc = lib3().gclaw3_ref_fill_ghosts(m, mx, my, mz, 2, _ip(np.array(bc_lower, np.int32)),
                                       _ip(np.array(bc_upper, np.int32)), _dp(qf), _dp(qbc))
    if rc:
        raise ValueError(f"gclaw3_ref_fill_ghosts failed: {rc}")
    return qbc


def step3(rp, pd, q, dx, dy, dz, dt, bc_lower, bc_upper, order=2, tw=22, mthlim=(4,) * 4,
          nthreads=1):
    """Ghost fill + unsplit 3D step; returns (qnew, cfl)."""
    m, mx, my, mz = q.shape
    qf = np.asfortranarray(q, dtype=np.float64)
    qout = np.zeros_like(qf, order="F")
    cfl = np.zeros(1)
    lim = np.zeros(5, np.int32)
    lim[:len(mthlim)] = mthlim
    rc = lib3().gclaw3_ref_step(rp, _dp(_pd(pd)), mx, my, mz, _dp(qf), _dp(qout), dx, dy, dz,
                                dt, order, tw, _ip(lim), _ip(np.array(bc_lower, np.int32)),
                                _ip(np.array(bc_upper, np.int32)), _dp(cfl), nthreads)
    if rc < 0:
        raise ValueError(f"gclaw3_ref_step failed: {rc}")
    if rc:
        raise FloatingPointError(f"gclaw3_ref_step: non-physical state ({rc})")
    return qout, float(cfl[0])


def rpn3(rp, pd, d, ql, qr):
    """One 3D Riemann problem along axis d: (waves (mw, m), s, amdq, apdq, rc)."""
    m, mw = SHAPES3[rp]
    ql = np.ascontiguousarray(ql, dtype=np.float64)
    qr = np.ascontiguousarray(qr, dtype=np.float64)
    W, s, am, ap = np.zeros(mw * m), np.zeros(mw), np.zeros(m), np.zeros(m)
    rc = lib3().gclaw3_ref_rpn3(rp, _dp(_pd(pd)), d, _dp(ql), _dp(qr), _dp(W), _dp(s), _dp(am),
                                _dp(ap))
    return W.reshape(mw, m), s, am, ap, rc


def step3_bc(rp, pd, qbc, dx, dy, dz, dt, order=2, tw=22, mthlim=(4,) * 4, nthreads=1):
    """The 3D step on a ghost-filled (m, mx+4, my+4, mz+4) array."""
    m = qbc.shape[0]
    mx, my, mz = (s - 4 for s in qbc.shape[1:])
    qf = np.asfortranarray(qbc, dtype=np.float64)
    qout = np.zeros_like(qf, order="F")
    cfl = np.zeros(1)
    lim = np.zeros(5, np.int32)
    lim[:len(mthlim)] = mthlim
    rc = lib3().gclaw3_ref_step3(rp, _dp(_pd(pd)), mx, my, mz, _dp(qf), _dp(qout), dx, dy, dz,
                                 dt, order, tw, _ip(lim), _dp(cfl), nthreads)
    if rc:
        raise ValueError(f"gclaw3_ref_step3 failed: {rc}")
    return qout, float(cfl[0])


def step3_split(rp, pd, q, dx, dy, dz, dt, bc_lower, bc_upper, order=2, mthlim=(4,) * 4,
                nthreads=1):
    """PyClaw's dimensionally split 3D step (x, y, z sweeps, boundary
    conditions before each); returns (qnew, cfl)."""
    m, mx, my, mz = q.shape
    qf = np.asfortranarray(q, dtype=np.float64)
    qout = np.zeros_like(qf, order="F")
    cfl = np.zeros(1)
    lim = np.zeros(5, np.int32)
    lim[:len(mthlim)] = mthlim
    rc = lib3().gclaw3_ref_step_split(rp, _dp(_pd(pd)), mx, my, mz, _dp(qf), _dp(qout), dx, dy,
                                      dz, dt, order, _ip(lim), _ip(np.array(bc_lower, np.int32)),
                                      _ip(np.array(bc_upper, np.int32)), _dp(cfl), nthreads)
    if rc < 0:
        raise ValueError(f"gclaw3_ref_step_split failed: {rc}")
    if rc:
        raise FloatingPointError(f"gclaw3_ref_step_split: non-physical state ({rc})")
    return qout, float(cfl[0])
