"""ClawSolver2D with a CUDA ``kernel_language`` backend.

Mirrors the attribute API of PyClaw's ClawSolver2D (upstream
pyclaw/src/pyclaw/classic/solver.py and pyclaw/src/pyclaw/solver.py; the
pyclaw submodule is empty in the mounted clawpack 5.14.0 tree,
meson.build:64): ``rp``, ``limiters``, ``order``, ``transverse_waves``,
``dimensional_split``, ``cfl_max``, ``cfl_desired``, ``dt_initial``,
``dt_max``, ``dt_variable``, ``max_steps``, ``bc_lower``, ``bc_upper``,
``num_ghost``, ``step()``, ``evolve_to_time()``, ``status``, ``cfl``.

The step itself runs in libgclaw.so on the GPU; there is no CPU path.  With
``dimensional_split = True`` (PyClaw's default) takes Godunov-split steps,
an x-sweep and then a y-sweep without transverse waves
(``transverse_waves`` is ignored); ``False`` takes the unsplit step.  With
``device_control = True`` (default) the evolve_to_time loop (dt choice, CFL
rejection, landing on tend) runs on the device as well, so the host only
waits once per batch of ``batch`` step launches.
"""
from __future__ import annotations

import logging
import math

import numpy as np

from .. import _lib
from ..device import DeviceProblem, DeviceProblem3, make_solver3_struct, make_solver_struct
from .limiters import tvd


class BC:
    """Boundary-condition ids (pyclaw.BC)."""
    custom = 0
    extrap = 1
    periodic = 2
    wall = 3


class CFLReduction:
    """Holds the Courant number of the last step (PyClaw's ``solver.cfl``)."""

    def __init__(self):
        self._v = 0.0

    def get_cached_max(self):
        return self._v

    def update_global_max(self, v):
        self._v = float(v)

    set_local_max = update_global_max


class ClawSolver2D:
    no_trans = 0
    trans_inc = 1
    trans_cor = 2

    def __init__(self, riemann_solver=None, claw_package=None):
        self.rp = None
        self.num_eqn = None
        self.num_waves = None
        if riemann_solver is not None:
            self.rp = riemann_solver
            self.num_eqn = riemann_solver.num_eqn
            self.num_waves = riemann_solver.num_waves
        self.num_dim = 2
        self.num_ghost = 2
        self.dimensional_split = True
        self.transverse_waves = self.trans_inc
        self.order = 2
        self.limiters = tvd.minmod
        self.fwave = False
        self.source_split = 1
        self.step_source = None
        self.before_step = None
        self.kernel_language = "CUDA"
        self.precision = "fp64"
        self.dt_initial = 0.1
        self.dt_max = 1e99
        self.cfl_max = 1.0
        self.cfl_desired = 0.9
        self.max_steps = 10000
        self.dt_variable = True
        self.bc_lower = [None, None]
        self.bc_upper = [None, None]
        self.aux_bc_lower = [None, None]
        self.aux_bc_upper = [None, None]
        self.reflect_index = [1, 2]
        self.device_control = True
        self.batch = 32
        self.dt = self.dt_initial
        self.cfl = CFLReduction()
        self.status = {"cflmax": -np.inf, "dtmin": np.inf, "dtmax": -np.inf, "numsteps": 0}
        self.logger = logging.getLogger("pyclaw.solver")
        self._is_set_up = False
        self._dev = None
        self._dev_key = None

    # ------------------------------------------------------------------ setup
    @property
    def _mthlim(self):
        lim = self.limiters
        if not isinstance(lim, (list, tuple)):
            lim = [lim]
        lim = list(lim)
        if len(lim) == 1:
            lim = lim * self.num_waves
        if len(lim) != self.num_waves:
            raise ValueError("Length of solver.limiters is not equal to 1 or to solver.num_waves")
        return [int(x) for x in lim]

    def _problem_data(self, state):
        pd = state.problem_data
        rp = self.rp.rp_id
        if rp == _lib.RP_ACOUSTICS_2D:
            rho = float(pd["rho"])
            bulk = float(pd["bulk"])
            cc = float(pd["cc"]) if "cc" in pd else math.sqrt(bulk / rho)
            zz = float(pd["zz"]) if "zz" in pd else rho * cc
            return [rho, bulk, cc, zz]
        if rp in (_lib.RP_SHALLOW_ROE_WITH_EFIX_2D, _lib.RP_SHALLOW_BATHYMETRY_FWAVE_2D):
            return [float(pd["grav"])]
        if rp == _lib.RP_VC_ACOUSTICS_2D:
            return []  # the medium is in state.aux
        return [float(pd["gamma"]), 1.0 if pd.get("efix", True) else 0.0]

    def _check_options(self, state):
        if self.rp is None:
            raise ValueError("solver.rp is not set")
        if getattr(self.rp, "num_dim", 2) != 2:
            raise ValueError(f"{self.rp.name} is not a 2D Riemann solver")
        if self.kernel_language != "CUDA":
            raise NotImplementedError(
                f"kernel_language={self.kernel_language!r}: this framework provides the 'CUDA' "
                "backend only")
        rp_fwave = getattr(self.rp, "fwave", False)
        if bool(self.fwave) != rp_fwave:
            raise ValueError(f"{self.rp.name} needs solver.fwave = {rp_fwave}")
        if self.step_source is not None and self.source_split not in (1, 2):
            raise ValueError("solver.source_split must be 1 (Godunov) or 2 (Strang)")
        if self.num_ghost != 2:
            raise ValueError("num_ghost must be 2")
        need_aux = getattr(self.rp, "num_aux", 0)
        capa = getattr(state, "index_capa", -1)
        if capa >= 0:
            if capa != need_aux:
                raise NotImplementedError(
                    f"the capacity must be the aux field after {self.rp.name}'s own "
                    f"(state.index_capa = {need_aux})")
            if self.precision != "fp64":
                raise NotImplementedError("a capacity function needs solver.precision = 'fp64'")
            need_aux += 1
        if state.num_aux != need_aux:
            raise ValueError(f"{self.rp.name} needs num_aux = {need_aux}, the state has "
                             f"{state.num_aux}")
        if need_aux:
            if state.aux is None:
                raise ValueError("state.aux is not set")
            if self.dimensional_split:
                raise NotImplementedError("dimensional splitting with an aux array is not "
                                          "supported; set solver.dimensional_split = False")
            for b in list(self.aux_bc_lower) + list(self.aux_bc_upper):
                if b is None:
                    raise ValueError("aux boundary conditions are not set (solver.aux_bc_lower, "
                                     "solver.aux_bc_upper)")
                if b == BC.custom:
                    raise NotImplementedError("BC.custom is not supported by the CUDA backend")
        for b in list(self.bc_lower) + list(self.bc_upper):
            if b is None:
                raise ValueError("boundary conditions are not set")
            if b == BC.custom:
                raise NotImplementedError("BC.custom is not supported by the CUDA backend")
        if self.precision not in ("fp64", "fp32"):
            raise ValueError("solver.precision must be 'fp64' or 'fp32'")

    def solver_struct(self, state):
        """The gclaw_solver C struct for this solver and grid."""
        self._check_options(state)
        g = state.grid
        mx, my = g.num_cells
        dx, dy = g.delta
        prec = _lib.PREC_FP64 if self.precision == "fp64" else _lib.PREC_FP32_BULK
        abl = self.aux_bc_lower if state.num_aux else (1, 1)
        abu = self.aux_bc_upper if state.num_aux else (1, 1)
        capa = getattr(state, "index_capa", -1)
        return make_solver_struct(self.rp.rp_id, mx, my, dx, dy, self.bc_lower, self.bc_upper,
                                  self._mthlim, self.order, self.transverse_waves, prec,
                                  self._problem_data(state), abl, abu,
                                  capa + 1 if capa >= 0 else 0)

    def setup(self, solution):
        self._check_options(solution.state)
        self.dt = self.dt_initial
        self.status = {"cflmax": -np.inf, "dtmin": np.inf, "dtmax": -np.inf, "numsteps": 0}
        self._is_set_up = True

    def _device(self, state):
        s = self.solver_struct(state)
        split = bool(self.dimensional_split)
        key = (bytes(s), split)
        if self._dev is None or self._dev_key != key:
            self._dev = DeviceProblem(s, split=split, aux=state.aux if state.num_aux else None)
            self._dev_key = key
        elif state.num_aux:
            self._dev.set_aux(state.aux)  # the caller may have changed the medium
        return self._dev

    # ------------------------------------------------------------------ stepping
    def step_hyperbolic(self, solution):
        """One hyperbolic step of size self.dt: the fused ghost fill + classic
        step on the GPU; sets state.q and returns the Courant number."""
        state = solution.state
        dev = self._device(state)
        dev.upload(state.q, 0)
        dev.step(self.dt, src=0)
        c = dev.read_ctrl()
        _lib.check(c.status, "step")
        self.cfl.update_global_max(c.cfl)
        state.q = dev.download(1)
        return c.cfl

    def step(self, solution, take_one_step=False, tstart=None, tend=None):
        """One step of size self.dt with PyClaw's source splitting:
        step_source(solver, state, dt) after the hyperbolic step
        (source_split 1, Godunov) or half steps before and after it
        (source_split 2, Strang); sets state.q and self.cfl."""
        state = solution.state
        if self.step_source is not None and self.source_split == 2:
            self.step_source(self, state, self.dt / 2.0)
        self.step_hyperbolic(solution)
        if self.step_source is not None:
            self.step_source(self, state, self.dt if self.source_split == 1 else self.dt / 2.0)
        return True

    def evolve_to_time(self, solution, tend=None):
        """Advance solution to tend with PyClaw's variable-dt rules.  With
        tend=None a single step is taken (PyClaw's take_one_step)."""
        if not self._is_set_up:
            self.setup(solution)
        if tend is None:
            return self._evolve(solution, math.inf, max_accepted=1)
        return self._evolve(solution, float(tend), max_accepted=-1)

    def evolve_steps(self, solution, nsteps):
        """Advance by exactly ``nsteps`` accepted steps (no end time)."""
        if not self._is_set_up:
            self.setup(solution)
        return self._evolve(solution, math.inf, max_accepted=int(nsteps))

    def _evolve(self, solution, tend, max_accepted):
        state = solution.state
        if self.step_source is not None or self.before_step is not None:
            return self._evolve_hooked(solution, tend, max_accepted)
        dev = self._device(state)
        dev.upload(state.q, 0)
        if self.device_control:
            c = dev.evolve(solution.t, self.dt, tend, cfl_max=self.cfl_max,
                           cfl_desired=self.cfl_desired, dt_max=self.dt_max,
                           max_steps=self.max_steps, max_accepted=max_accepted,
                           dt_variable=self.dt_variable, batch=self.batch)
            t, dt, parity = c.t, c.dt, c.parity
            numsteps, cflmax, cfl = c.numsteps, c.cflmax, c.cfl
            dtmin, dtmax, status = c.dtmin, c.dtmax, c.status
        else:
            t, dt, parity, numsteps, cflmax, cfl, dtmin, dtmax, status = self._host_loop(
                dev, solution.t, self.dt, tend, max_accepted)
        state.q = dev.download(parity)
        solution.t = t
        self.dt = dt
        self.cfl.update_global_max(cfl)
        self.status["numsteps"] += numsteps
        if numsteps:
            self.status["cflmax"] = max(self.status["cflmax"], cflmax)
        self.status["dtmin"] = min(self.status["dtmin"], dtmin)
        self.status["dtmax"] = max(self.status["dtmax"], dtmax)
        self.logger.debug("evolve to t=%g: %d steps, last dt=%g, cfl=%g", t, numsteps, dt, cfl)
        _lib.check(status, "evolve_to_time")
        return self.status

    def _evolve_hooked(self, solution, tend, max_accepted):
        """evolve_to_time with Python hooks (before_step, step_source): the
        hooks see state.q as a host array, so every attempt runs on the host:
        before_step, step() (source splitting around the GPU step), then the
        CFL check, which restores the state of the start of the step on
        rejection (upstream pyclaw/src/pyclaw/solver.py)."""
        state = solution.state
        t, dt = solution.t, self.dt
        tstart = t
        numsteps = 0
        cflmax = 0.0
        dtmin = dtmax = dt
        status = _lib.MAX_STEPS
        for _ in range(self.max_steps):
            if t + dt > tend and tstart < tend:
                dt = tend - t
            if tend - t - dt < 1.0e-14 * t:
                dt = tend - t
            q_backup = state.q.copy(order="F")
            state.t = t
            if self.before_step is not None:
                self.before_step(self, state)
            self.dt = dt
            self.step(solution)
            cfl = self.cfl.get_cached_max()
            if cfl <= self.cfl_max:
                cflmax = max(cfl, cflmax)
                numsteps += 1
                t = t + dt if self.dt_variable else tstart + numsteps * dt
            else:
                state.q = q_backup
                if not self.dt_variable:
                    status = _lib.CFL_FIXED_DT
                    break
            if t >= tend or (max_accepted >= 0 and numsteps >= max_accepted):
                status = _lib.OK
                break
            if self.dt_variable:
                if cfl > 0.0:
                    dt = min(self.dt_max, dt * self.cfl_desired / cfl)
                    dtmin = min(dt, dtmin)
                    dtmax = max(dt, dtmax)
                else:
                    dt = self.dt_max
        solution.t = t
        state.t = t
        self.dt = dt
        self.status["numsteps"] += numsteps
        if numsteps:
            self.status["cflmax"] = max(self.status["cflmax"], cflmax)
        self.status["dtmin"] = min(self.status["dtmin"], dtmin)
        self.status["dtmax"] = max(self.status["dtmax"], dtmax)
        _lib.check(status, "evolve_to_time")
        return self.status

    def _host_loop(self, dev, t, dt, tend, max_accepted):
        """The evolve_to_time loop on the host: one step launch and one CFL
        read-back per attempt (the per-step path of the reference)."""
        tstart = t
        parity = 0
        numsteps = attempts = 0
        cflmax, cfl = 0.0, 0.0
        dtmin = dtmax = dt
        for _ in range(self.max_steps):
            if t + dt > tend and tstart < tend:
                dt = tend - t
            if tend - t - dt < 1.0e-14 * t:
                dt = tend - t
            dev.step(dt, src=parity)
            c = dev.read_ctrl()
            attempts += 1
            cfl = c.cfl
            if c.status:
                return t, dt, parity, numsteps, cflmax, cfl, dtmin, dtmax, c.status
            if cfl <= self.cfl_max:
                cflmax = max(cfl, cflmax)
                numsteps += 1
                t = t + dt if self.dt_variable else tstart + numsteps * dt
                parity ^= 1
            elif not self.dt_variable:
                return t, dt, parity, numsteps, cflmax, cfl, dtmin, dtmax, _lib.CFL_FIXED_DT
            if t >= tend or (max_accepted >= 0 and numsteps >= max_accepted):
                return t, dt, parity, numsteps, cflmax, cfl, dtmin, dtmax, _lib.OK
            if self.dt_variable:
                if cfl > 0.0:
                    dt = min(self.dt_max, dt * self.cfl_desired / cfl)
                    dtmin = min(dt, dtmin)
                    dtmax = max(dt, dtmax)
                else:
                    dt = self.dt_max
        return t, dt, parity, numsteps, cflmax, cfl, dtmin, dtmax, _lib.MAX_STEPS


class ClawSolver3D(ClawSolver2D):
    """PyClaw's ClawSolver3D (upstream pyclaw/src/pyclaw/classic/solver.py)
    on the CUDA backend: the unsplit 3D step of gclaw3.h.

    ``transverse_waves`` takes ClawSolver3D's values: 0, 10 / 11
    (``trans_inc``: transverse propagation of the increment waves, without /
    with the corner terms) and 20 / 22 (``trans_cor``: also of the correction
    waves).  ``dimensional_split = True`` (the default) takes x-, y- and
    z-sweeps in turn without transverse terms; ``False`` the unsplit step.
    Without aux arrays, in FP64 or FP32-bulk (``precision``)."""
    no_trans = 0
    trans_inc = 11
    trans_cor = 22

    def __init__(self, riemann_solver=None, claw_package=None):
        super().__init__(riemann_solver, claw_package)
        self.num_dim = 3
        self.transverse_waves = self.trans_cor
        self.bc_lower = [None, None, None]
        self.bc_upper = [None, None, None]
        self.aux_bc_lower = [None, None, None]
        self.aux_bc_upper = [None, None, None]
        self.reflect_index = [1, 2, 3]

    def _problem_data(self, state):
        pd = state.problem_data
        if self.rp.rp_id == _lib.RP3_EULER_3D:
            return [float(pd["gamma"])]
        rho = float(pd["rho"])
        bulk = float(pd["bulk"])
        cc = float(pd["cc"]) if "cc" in pd else math.sqrt(bulk / rho)
        zz = float(pd["zz"]) if "zz" in pd else rho * cc
        return [rho, bulk, cc, zz]

    def _check_options(self, state):
        if self.rp is None:
            raise ValueError("solver.rp is not set")
        if getattr(self.rp, "num_dim", 2) != 3:
            raise ValueError(f"{self.rp.name} is not a 3D Riemann solver")
        if self.kernel_language != "CUDA":
            raise NotImplementedError(
                f"kernel_language={self.kernel_language!r}: this framework provides the 'CUDA' "
                "backend only")
        if self.fwave:
            raise ValueError(f"{self.rp.name} needs solver.fwave = False")
        if state.num_aux or getattr(state, "index_capa", -1) >= 0:
            raise NotImplementedError("3D steps with aux arrays are not supported")
        if self.num_ghost != 2:
            raise ValueError("num_ghost must be 2")
        if self.transverse_waves not in (0, 10, 11, 20, 22):
            raise NotImplementedError("transverse_waves must be 0, 10, 11, 20 or 22")
        for b in list(self.bc_lower) + list(self.bc_upper):
            if b is None:
                raise ValueError("boundary conditions are not set")
            if b == BC.custom:
                raise NotImplementedError("BC.custom is not supported by the CUDA backend")
        if self.precision not in ("fp64", "fp32"):
            raise ValueError("solver.precision must be 'fp64' or 'fp32'")
        if self.step_source is not None and self.source_split not in (1, 2):
            raise ValueError("solver.source_split must be 1 (Godunov) or 2 (Strang)")

    def solver_struct(self, state):
        """The gclaw3_solver C struct for this solver and grid."""
        self._check_options(state)
        g = state.grid
        mx, my, mz = g.num_cells
        dx, dy, dz = g.delta
        return make_solver3_struct(self.rp.rp_id, mx, my, mz, dx, dy, dz, self.bc_lower,
                                   self.bc_upper, self._mthlim, self.order,
                                   self.transverse_waves,
                                   _lib.PREC_FP64 if self.precision == "fp64"
                                   else _lib.PREC_FP32_BULK, self._problem_data(state))

    def _device(self, state):
        s = self.solver_struct(state)
        split = bool(self.dimensional_split)
        key = (bytes(s), split)
        if self._dev is None or self._dev_key != key:
            self._dev = DeviceProblem3(s, split=split)
            self._dev_key = key
        return self._dev
