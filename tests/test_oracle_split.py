"""Known answers for the dimensionally split step of the oracle
(gclaw_ref_step_split: boundary conditions, x-sweep, boundary conditions,
y-sweep, no transverse waves).

Wall boundaries conserve the conserved quantities; data uniform in y with
no y-momentum (or uniform in x with no x-momentum) make one sweep the
identity, so the split step equals the unsplit step with transverse_waves
0 bit for bit; otherwise the two differ (the order of the sweeps matters)."""
import numpy as np
import pytest

from oracle import ref
from tests.helpers import PD, random_state, rel_l1

RPS = [1, 2, 3]
CONSERVED = {1: [0], 2: [0, 1, 2], 3: [0, 3]}


@pytest.mark.parametrize("rp", RPS)
@pytest.mark.parametrize("lim", [1, 2, 4])
def test_wall_boundaries_conserve(rp, lim):
    rng = np.random.default_rng(rp * 10 + lim)
    q = random_state(rp, 23, 17, rng)
    if rp == 2:
        q[1:] = 0.0  # momentum is not conserved at walls; start at rest
    qn, cfl, rc = ref.step_split(rp, PD[rp], q, 0.04, 0.05, 0.004, [3, 3], [3, 3], 2, [lim] * 4)
    assert rc == 0 and cfl > 0
    for k in CONSERVED[rp] if rp != 2 else [0]:
        assert abs(qn[k].sum() - q[k].sum()) <= 1e-12 * np.abs(q[k]).sum()


def _uniform(rp, mx, my, along):
    rng = np.random.default_rng(7 + rp)
    line = random_state(rp, mx if along == "x" else my, 1, rng)[:, :, 0]
    q = np.empty((line.shape[0], mx, my), order="F")
    for k in range(line.shape[0]):
        q[k] = line[k][:, None] if along == "x" else line[k][None, :]
    # no momentum across the uniform direction
    if rp in (1, 2, 3):
        q[2 if along == "x" else 1] = 0.0
    if rp == 3:  # keep E consistent with the zeroed momentum
        rho, u, v = q[0], q[1] / q[0], q[2] / q[0]
        q[3] = 1.0 / 0.4 + 0.5 * rho * (u * u + v * v)
    return q


@pytest.mark.parametrize("rp", RPS)
@pytest.mark.parametrize("along", ["x", "y"])
def test_one_dimensional_data_reduces_to_the_unsplit_step(rp, along):
    """Data varying only along ``along`` (with the other momentum zero): the
    other sweep has zero waves, so the split step equals the unsplit step
    with transverse_waves 0 bit for bit, and so do the Courant numbers."""
    q = _uniform(rp, 31, 26, along)
    bcl, bcu = [1, 3], [3, 1]
    a, ca, ra = ref.step_split(rp, PD[rp], q, 0.03, 0.04, 0.003, bcl, bcu, 2, [4] * 4)
    b, cb, rb = ref.step(rp, PD[rp], q, 0.03, 0.04, 0.003, bcl, bcu, 2, 0, [4] * 4)
    assert ra == rb == 0
    assert np.array_equal(a, b)
    assert ca == cb


@pytest.mark.parametrize("rp", RPS)
def test_split_differs_from_unsplit_on_2d_data(rp):
    rng = np.random.default_rng(3)
    q = random_state(rp, 20, 18, rng)
    a, _, _ = ref.step_split(rp, PD[rp], q, 0.05, 0.05, 0.004, [1, 1], [1, 1], 2, [4] * 4)
    b, _, _ = ref.step(rp, PD[rp], q, 0.05, 0.05, 0.004, [1, 1], [1, 1], 2, 0, [4] * 4)
    assert 0.0 < rel_l1(a, b) < 0.1
