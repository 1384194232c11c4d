"""Initial and boundary data of the benchmark problems.

Each function returns a ``Workload`` describing one problem of the classic
2D path: solver, problem data, grid, boundary conditions, limiters, CFL
targets, the initial state q0 (num_eqn, mx, my) in Fortran order, and either
an end time or a number of accepted steps.  All data are synthetic and
seeded; no dataset is involved.

  acoustics_radial   2D acoustics, 200x200 on [-1,1]^2, rho=1, K=4 (c=2),
                     p = exp(-100 r^2), u=v=0, extrapolation BCs, MC limiter,
                     transverse_waves=2, CFL 0.9, t_final 0.6, 10 frames
  shallow_dam_break  shallow water Roe + entropy fix, 2048x2048 on
                     [-2.5,2.5]^2, g=1, h=2 for r<0.5 else 1, wall BCs, MC,
                     transverse_waves=2, CFL 0.9, 1000 steps
  euler_quadrants    2D Euler Roe 4-wave, gamma=1.4, 4096x4096 on [0,1]^2,
                     four quadrant states drawn from a seed (rho, p in
                     U[0.1,1.5], u, v in U[-1,1]), extrapolation BCs,
                     superbee, CFL 0.8, 500 steps
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .pyclaw.limiters import tvd
from .pyclaw.solver import BC

EULER_SEED = 20261204


@dataclass
class Workload:
    name: str
    rp_name: str
    rp_id: int
    problem_data: dict
    lower: tuple
    upper: tuple
    mx: int
    my: int
    q0: np.ndarray
    bc_lower: list
    bc_upper: list
    limiters: int
    order: int = 2
    transverse_waves: int = 2
    cfl_desired: float = 0.9
    cfl_max: float = 1.0
    dt_initial: float = 0.1
    tfinal: float = None
    nsteps: int = None
    num_output_times: int = 10
    meta: dict = field(default_factory=dict)

    @property
    def dx(self):
        return (self.upper[0] - self.lower[0]) / self.mx

    @property
    def dy(self):
        return (self.upper[1] - self.lower[1]) / self.my

    @property
    def num_eqn(self):
        return self.q0.shape[0]

    def pd_array(self):
        """problem_data in the gclaw_solver.problem_data layout."""
        pd = self.problem_data
        if self.rp_id == _lib.RP_ACOUSTICS_2D:
            return [pd["rho"], pd["bulk"], pd["cc"], pd["zz"]]
        if self.rp_id == _lib.RP_SHALLOW_ROE_WITH_EFIX_2D:
            return [pd["grav"]]
        return [pd["gamma"], 1.0 if pd.get("efix", True) else 0.0]

    @property
    def num_waves(self):
        return {_lib.RP_ACOUSTICS_2D: 2, _lib.RP_SHALLOW_ROE_WITH_EFIX_2D: 3,
                _lib.RP_EULER_4WAVE_2D: 4}[self.rp_id]

    def mthlim(self, num_waves=None):
        return [self.limiters] * (num_waves or self.num_waves)

    def solver_struct(self, precision=_lib.PREC_FP64):
        """The gclaw_solver C struct of this workload."""
        from .device import make_solver_struct

        return make_solver_struct(self.rp_id, self.mx, self.my, self.dx, self.dy,
                                  self.bc_lower, self.bc_upper, self.mthlim(), self.order,
                                  self.transverse_waves, precision, self.pd_array())


def _centers(lower, upper, n):
    d = (upper - lower) / n
    return lower + (np.arange(n) + 0.5) * d


def acoustics_radial(mx=200, my=200):
    x = _centers(-1.0, 1.0, mx)
    y = _centers(-1.0, 1.0, my)
    X, Y = np.meshgrid(x, y, indexing="ij")
    rho, bulk = 1.0, 4.0
    cc = math.sqrt(bulk / rho)
    zz = rho * cc
    q = np.zeros((3, mx, my), order="F")
    q[0] = np.exp(-100.0 * (X * X + Y * Y))
    return Workload("acoustics_radial", "acoustics_2D", _lib.RP_ACOUSTICS_2D,
                    dict(rho=rho, bulk=bulk, cc=cc, zz=zz), (-1.0, -1.0), (1.0, 1.0), mx, my, q,
                    [BC.extrap, BC.extrap], [BC.extrap, BC.extrap], tvd.MC, cfl_desired=0.9,
                    dt_initial=0.1, tfinal=0.6, num_output_times=10)


def shallow_dam_break(mx=2048, my=2048, nsteps=1000):
    x = _centers(-2.5, 2.5, mx)
    y = _centers(-2.5, 2.5, my)
    X, Y = np.meshgrid(x, y, indexing="ij")
    q = np.zeros((3, mx, my), order="F")
    q[0] = np.where(np.sqrt(X * X + Y * Y) < 0.5, 2.0, 1.0)
    g = 1.0
    dx = 5.0 / mx
    # first dt from the initial wave speed sqrt(g h_max), so no attempt is rejected
    dt0 = 0.9 * dx / math.sqrt(g * 2.0)
    return Workload("shallow_dam_break", "shallow_roe_with_efix_2D",
                    _lib.RP_SHALLOW_ROE_WITH_EFIX_2D, dict(grav=g), (-2.5, -2.5), (2.5, 2.5), mx,
                    my, q, [BC.wall, BC.wall], [BC.wall, BC.wall], tvd.MC, cfl_desired=0.9,
                    dt_initial=dt0, nsteps=nsteps)


def euler_quadrant_states(seed=EULER_SEED):
    """Four (rho, u, v, p) states, quadrants ordered (x<.5,y<.5), (x>.5,y<.5),
    (x<.5,y>.5), (x>.5,y>.5)."""
    rng = np.random.default_rng(seed)
    st = []
    for _ in range(4):
        rho = rng.uniform(0.1, 1.5)
        u = rng.uniform(-1.0, 1.0)
        v = rng.uniform(-1.0, 1.0)
        p = rng.uniform(0.1, 1.5)
        st.append((rho, u, v, p))
    return st


def euler_quadrants(mx=4096, my=4096, nsteps=500, seed=EULER_SEED, gamma=1.4):
    x = _centers(0.0, 1.0, mx)
    y = _centers(0.0, 1.0, my)
    X, Y = np.meshgrid(x, y, indexing="ij")
    states = euler_quadrant_states(seed)
    q = np.zeros((4, mx, my), order="F")
    quad = (X > 0.5).astype(int) + 2 * (Y > 0.5).astype(int)
    smax = 0.0
    for k, (rho, u, v, p) in enumerate(states):
        msk = quad == k
        q[0][msk] = rho
        q[1][msk] = rho * u
        q[2][msk] = rho * v
        q[3][msk] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
        smax = max(smax, max(abs(u), abs(v)) + math.sqrt(gamma * p / rho))
    dt0 = 0.8 * min(1.0 / mx, 1.0 / my) / smax
    return Workload("euler_quadrants", "euler_4wave_2D", _lib.RP_EULER_4WAVE_2D,
                    dict(gamma=gamma, efix=True), (0.0, 0.0), (1.0, 1.0), mx, my, q,
                    [BC.extrap, BC.extrap], [BC.extrap, BC.extrap], tvd.superbee,
                    cfl_desired=0.8, dt_initial=dt0, nsteps=nsteps,
                    meta=dict(seed=seed, states=states))


def make_claw(w: Workload, precision="fp64"):
    """A pyclaw Controller set up for workload ``w``."""
    from . import riemann
    from .pyclaw import ClawSolver2D, Controller, Dimension, Domain, Solution, State

    solver = ClawSolver2D(getattr(riemann, w.rp_name))
    solver.dimensional_split = False
    solver.transverse_waves = w.transverse_waves
    solver.order = w.order
    solver.limiters = w.limiters
    solver.cfl_desired = w.cfl_desired
    solver.cfl_max = w.cfl_max
    solver.dt_initial = w.dt_initial
    solver.bc_lower = list(w.bc_lower)
    solver.bc_upper = list(w.bc_upper)
    solver.precision = precision
    x = Dimension(w.lower[0], w.upper[0], w.mx, name="x")
    y = Dimension(w.lower[1], w.upper[1], w.my, name="y")
    domain = Domain([x, y])
    state = State(domain, solver.num_eqn)
    state.problem_data.update(w.problem_data)
    state.q = w.q0
    claw = Controller()
    claw.solution = Solution(state, domain)
    claw.solver = solver
    if w.tfinal is not None:
        claw.tfinal = w.tfinal
        claw.num_output_times = w.num_output_times
    return claw


BATCH_SEED = 20261205


@dataclass
class Ensemble:
    """Many independent shallow-water problems on [0,1]^2 with wall BCs."""
    shapes: list
    deltas: list
    params: list   # per problem (a, b, x0, y0)
    dt0: np.ndarray
    grav: float = 1.0
    cfl_desired: float = 0.9
    cfl_max: float = 1.0
    nsteps: int = 200
    seed: int = BATCH_SEED

    @property
    def cells(self):
        return int(sum(a * b for a, b in self.shapes))

    def q0(self, p):
        """Initial state (3, mx, my) of problem p: h = 1 + a exp(-b |x - x0|^2)."""
        mx, my = self.shapes[p]
        a, b, x0, y0 = self.params[p]
        X, Y = np.meshgrid(_centers(0.0, 1.0, mx), _centers(0.0, 1.0, my), indexing="ij")
        q = np.zeros((3, mx, my), order="F")
        q[0] = 1.0 + a * np.exp(-b * ((X - x0) ** 2 + (Y - y0) ** 2))
        return q


def batched_ensemble(nprob=4096, smin=32, smax=512, nsteps=200, seed=BATCH_SEED):
    """4096 shallow-water problems, square grids with side log-uniform in
    [smin, smax]; h = 1 + a exp(-b |x-x0|^2), a in U[0.05, 0.5], b in
    U[20, 200], x0 uniform in the domain; hu = hv = 0; first dt of each
    problem from its own initial wave speed at CFL 0.9."""
    rng = np.random.default_rng(seed)
    sides = np.rint(np.exp(rng.uniform(math.log(smin), math.log(smax), nprob))).astype(int)
    a = rng.uniform(0.05, 0.5, nprob)
    b = rng.uniform(20.0, 200.0, nprob)
    x0 = rng.uniform(0.0, 1.0, (nprob, 2))
    shapes = [(int(s), int(s)) for s in sides]
    deltas = [(1.0 / s, 1.0 / s) for s in sides]
    params = [(float(a[p]), float(b[p]), float(x0[p, 0]), float(x0[p, 1])) for p in range(nprob)]
    dt0 = np.array([0.9 * (1.0 / s) / math.sqrt(1.0 * (1.0 + ap)) for s, ap in zip(sides, a)])
    return Ensemble(shapes, deltas, params, dt0, nsteps=nsteps, seed=seed)


def make_batch(e: Ensemble, precision=_lib.PREC_FP32_BULK, device=None):
    """A BatchSolver loaded with ensemble e's initial states and controls."""
    from .batch import BatchSolver

    bs = BatchSolver(_lib.RP_SHALLOW_ROE_WITH_EFIX_2D, e.shapes, e.deltas, [BC.wall, BC.wall],
                     [BC.wall, BC.wall], [tvd.MC] * 3, [e.grav], precision=precision,
                     device=device)
    host = bs.pinned_host_buffer()
    for p in range(len(e.shapes)):
        bs.pack(host, p, e.q0(p))
    bs.upload(host)
    bs.ctrl_init(e.dt0, cfl_max=e.cfl_max, cfl_desired=e.cfl_desired, max_accepted=e.nsteps,
                 max_steps=10 * e.nsteps)
    return bs


ADJOINT_SEED = 20261206


@dataclass
class AdjointProblem:
    """Least-squares fit of gauge series: shallow water on [0,1]^2, wall BCs,
    MC limiter, transverse_waves 2; h0 = 1 + sum of 16 seeded Gaussians of
    amplitude <= 0.2; loss = sum over steps and 64 gauge cells of
    (h - target)^2, targets from a run of a second seeded initial surface."""
    mx: int
    my: int
    nsteps: int
    checkpoint_every: int
    h0: np.ndarray
    h_true: np.ndarray
    gauges: np.ndarray  # (64, 2) cell indices (i, j)
    grav: float = 1.0
    cfl_desired: float = 0.9
    limiter: int = tvd.MC

    @property
    def dx(self):
        return 1.0 / self.mx

    def q0(self, h=None):
        q = np.zeros((3, self.mx, self.my), order="F")
        q[0] = self.h0 if h is None else h
        return q

    def solver_struct(self, precision=_lib.PREC_FP64):
        from .device import make_solver_struct

        return make_solver_struct(_lib.RP_SHALLOW_ROE_WITH_EFIX_2D, self.mx, self.my,
                                  1.0 / self.mx, 1.0 / self.my, [BC.wall, BC.wall],
                                  [BC.wall, BC.wall], [self.limiter] * 3, 2, 2, precision,
                                  [self.grav])

    @property
    def dt0(self):
        return self.cfl_desired * self.dx / math.sqrt(self.grav * float(self.h0.max()))


def _bumps(rng, mx, my, n=16, amp=0.2):
    X, Y = np.meshgrid(_centers(0.0, 1.0, mx), _centers(0.0, 1.0, my), indexing="ij")
    h = np.ones((mx, my))
    for _ in range(n):
        a = rng.uniform(0.0, amp)
        b = rng.uniform(50.0, 300.0)
        x0, y0 = rng.uniform(0.1, 0.9, 2)
        h += a * np.exp(-b * ((X - x0) ** 2 + (Y - y0) ** 2))
    return h


def adjoint_problem(mx=1024, my=None, nsteps=500, checkpoint_every=23, seed=ADJOINT_SEED,
                    limiter=tvd.MC):
    my = my or mx
    rng = np.random.default_rng(seed)
    h0 = _bumps(rng, mx, my)
    h_true = _bumps(rng, mx, my)
    gauges = np.stack([rng.integers(0, mx, 64), rng.integers(0, my, 64)], axis=1)
    return AdjointProblem(mx, my, nsteps, checkpoint_every, h0, h_true, gauges, limiter=limiter)


@dataclass
class Workload3:
    """A 3D problem: acoustics_3D on a cube, state (4, n, n, n)."""
    name: str
    n: int
    delta: tuple
    q0: np.ndarray
    problem_data: list
    bc_lower: list
    bc_upper: list
    dt_initial: float
    cfl_desired: float = 0.9
    cfl_max: float = 1.0

    rp_id: int = _lib.RP3_ACOUSTICS_3D
    num_waves: int = 2

    def solver_struct(self, order=2, tw=22, lim=tvd.MC, precision=_lib.PREC_FP64):
        from .device import make_solver3_struct

        return make_solver3_struct(self.rp_id, self.n, self.n, self.n, *self.delta,
                                   self.bc_lower, self.bc_upper, [lim] * self.num_waves, order,
                                   tw, precision, self.problem_data)


def acoustics_3d_pulse(n=192):
    """A Gaussian pressure pulse off the centre of [-1, 1]^3 between walls;
    rho = 1, bulk = 4 (c = 2), MC limiter, transverse_waves 22."""
    x = _centers(-1.0, 1.0, n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    q = np.zeros((4, n, n, n), order="F")
    q[0] = np.exp(-40.0 * ((X - 0.2) ** 2 + (Y + 0.1) ** 2 + Z ** 2))
    h = 2.0 / n
    # first dt from the sound speed, so no attempt is rejected
    return Workload3("acoustics_3d_pulse", n, (h, h, h), q, [1.0, 4.0, 2.0, 2.0],
                     [BC.wall] * 3, [BC.wall] * 3, dt_initial=0.9 * h / 2.0)


EULER3D_SEED = 20261207


def euler_3d_octants(n=128, seed=EULER3D_SEED, gamma=1.4):
    """Eight constant states in the octants of [0, 1]^3 split at the centre
    (rho, p ~ U[0.5, 1.5], velocity components ~ U[-0.5, 0.5], seeded),
    extrapolation boundaries: the 3D analogue of the four-quadrant problem."""
    rng = np.random.default_rng(seed)
    q = np.zeros((5, n, n, n), order="F")
    h = n // 2
    for o in range(8):
        sl = tuple(slice(0, h) if not (o >> k) & 1 else slice(h, n) for k in range(3))
        rho = rng.uniform(0.5, 1.5)
        u = rng.uniform(-0.5, 0.5, size=3)
        p = rng.uniform(0.5, 1.5)
        q[(0,) + sl] = rho
        for k in range(3):
            q[(1 + k,) + sl] = rho * u[k]
        q[(4,) + sl] = p / (gamma - 1.0) + 0.5 * rho * float((u ** 2).sum())
    dx = 1.0 / n
    return Workload3("euler_3d_octants", n, (dx, dx, dx), q, [gamma], [BC.extrap] * 3,
                     [BC.extrap] * 3, dt_initial=0.2 * dx, cfl_desired=0.8,
                     rp_id=_lib.RP3_EULER_3D, num_waves=3)
