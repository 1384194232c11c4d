"""PyClaw's source-term splitting and before_step hook on the GPU solver:
step_source(solver, state, dt) after the hyperbolic step (source_split 1)
or as half steps around it (source_split 2), with the evolve_to_time rules
(a rejected attempt restores the state of the start of the step), against
the oracle's evolve with the same splitting."""
import math

import numpy as np
import pytest

from clawpack_gb300 import workloads
from tests.helpers import rel_l1

pytestmark = pytest.mark.gpu

K = 3.0  # damping rate of q_t = -K q


def damp(solver, state, dt):
    state.q = state.q * math.exp(-K * dt)


def oracle_frames(oracle, w, split, dt0):
    def step(q, dt):
        if split == 2:
            q = q * math.exp(-K * dt / 2.0)
        qn, cfl, rc = oracle.step(w.rp_id, w.pd_array(), q, w.dx, w.dy, dt, w.bc_lower,
                                  w.bc_upper, w.order, w.transverse_waves, w.mthlim(2),
                                  nthreads=8)
        assert rc == 0
        qn = qn * math.exp(-K * dt / (1.0 if split == 1 else 2.0))
        return qn, cfl

    q, t, dt = w.q0, 0.0, dt0
    frames = [q]
    for tout in np.linspace(0.0, w.tfinal, w.num_output_times + 1)[1:]:
        q, t, dt, _ = oracle.evolve(step, q, t, tout, dt, cfl_desired=w.cfl_desired,
                                    cfl_max=w.cfl_max)
        frames.append(q)
    return frames


@pytest.mark.parametrize("split", [1, 2])
def test_source_splitting_matches_oracle(cuda, oracle, split):
    w = workloads.acoustics_radial(80, 64)
    w.tfinal, w.num_output_times = 0.2, 2
    claw = workloads.make_claw(w)
    claw.solver.step_source = damp
    claw.solver.source_split = split
    calls = []
    claw.solver.before_step = lambda solver, state: calls.append(state.t)
    claw.run()
    oframes = oracle_frames(oracle, w, split, w.dt_initial)
    for k, (a, b) in enumerate(zip(claw.frames, oframes)):
        assert rel_l1(a.q, b) <= 1e-12, k
    # dt_initial = 0.1 is rejected once: before_step runs for every attempt
    assert len(calls) == claw.solver.status["numsteps"] + 1
    # the damping acted: the pulse decayed faster than without the source
    assert np.abs(claw.frames[-1].q[0]).max() < math.exp(-K * 0.15) * np.abs(w.q0[0]).max()
