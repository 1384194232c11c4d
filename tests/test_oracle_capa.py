"""Known answers for the capacity form of the step in the oracle (classic2's
mcapa: a capacity kappa per cell as the last aux field).

kappa = 1 gives the plain step to round-off (the capacity form groups the
flux differences before dividing by kappa); a uniform kappa = c equals the
plain step on cells c times larger in x and y; sum(kappa q) is conserved
with periodic boundaries; a constant state stays constant bit for bit; the
step commutes with the x/y transpose; capacity combines with the aux
solvers (a lake at rest stays at rest on a non-uniform grid; a constant
medium gives constant-coefficient acoustics)."""
import math

import numpy as np
import pytest

from oracle import ref
from tests.helpers import PD, random_state, rel_l1

BASE = [1, 2, 3]


def kappa(mx, my, rng):
    """A smooth positive capacity with a little noise, in [0.5, 2]."""
    x = (np.arange(mx)[:, None] + 0.5) / mx
    y = (np.arange(my)[None, :] + 0.5) / my
    k = 1.2 + 0.6 * np.sin(2 * math.pi * x) * np.cos(2 * math.pi * y) + 0.1 * rng.random((mx, my))
    return np.asfortranarray(k[None])


@pytest.mark.parametrize("rp", BASE)
@pytest.mark.parametrize("order,tw,lim", [(2, 2, 4), (2, 1, 1), (1, 0, 0)])
def test_unit_capacity_is_the_plain_step(rp, order, tw, lim):
    rng = np.random.default_rng(rp + 10 * tw)
    mx, my = 23, 19
    q = random_state(rp, mx, my, rng)
    aux = np.ones((1, mx, my), order="F")
    a, ca, ra = ref.step_aux(rp, PD[rp], q, aux, 0.04, 0.05, 0.002, [3, 1], [1, 3], [1, 1], [1, 1],
                             order, tw, [lim] * 4, mcapa=1)
    b, cb, rb = ref.step(rp, PD[rp], q, 0.04, 0.05, 0.002, [3, 1], [1, 3], order, tw, [lim] * 4)
    assert ra == rb == 0
    assert rel_l1(a, b) <= 1e-15
    assert ca == cb


@pytest.mark.parametrize("rp", BASE)
def test_uniform_capacity_scales_the_cells(rp):
    rng = np.random.default_rng(rp)
    mx, my = 21, 26
    q = random_state(rp, mx, my, rng)
    aux = np.full((1, mx, my), 2.0, order="F")
    a, ca, _ = ref.step_aux(rp, PD[rp], q, aux, 0.04, 0.05, 0.003, [1, 2], [1, 2], [1, 2], [1, 2],
                            2, 2, [4] * 4, mcapa=1)
    b, cb, _ = ref.step(rp, PD[rp], q, 0.08, 0.10, 0.003, [1, 2], [1, 2], 2, 2, [4] * 4)
    assert rel_l1(a, b) <= 1e-14
    assert math.isclose(ca, cb, rel_tol=1e-15)


@pytest.mark.parametrize("rp", BASE)
def test_capacity_weighted_sum_conserved(rp):
    rng = np.random.default_rng(20 + rp)
    mx, my = 30, 24
    q = random_state(rp, mx, my, rng)
    aux = kappa(mx, my, rng)
    out, cfl, rc = ref.step_aux(rp, PD[rp], q, aux, 0.03, 0.03, 0.001, [2, 2], [2, 2], [2, 2],
                                [2, 2], 2, 2, [4] * 4, mcapa=1)
    assert rc == 0
    for k in range(q.shape[0]):
        s0, s1 = (aux[0] * q[k]).sum(), (aux[0] * out[k]).sum()
        assert abs(s1 - s0) <= 1e-13 * np.abs(aux[0] * q[k]).sum(), k


@pytest.mark.parametrize("rp", BASE)
def test_constant_state_is_preserved(rp):
    rng = np.random.default_rng(30 + rp)
    mx, my = 17, 15
    q = random_state(rp, 1, 1, rng) * np.ones((1, mx, my))
    q = np.asfortranarray(q)
    aux = kappa(mx, my, rng)
    out, cfl, rc = ref.step_aux(rp, PD[rp], q, aux, 0.05, 0.05, 0.002, [1, 1], [1, 1], [1, 1],
                                [1, 1], 2, 2, [4] * 4, mcapa=1)
    assert rc == 0
    assert np.array_equal(out, q)


def test_courant_number_uses_the_cells_capacity():
    mx, my = 12, 10
    q = np.zeros((3, mx, my), order="F")
    q[0, :6] = 1.0  # a pressure jump at one x-edge: speeds -c and +c there
    aux = np.ones((1, mx, my), order="F")
    aux[0, 5] = 0.25  # the cell left of the jump is 4 times smaller
    _, cfl, _ = ref.step_aux(1, PD[1], q, aux, 0.1, 0.1, 0.01, [1, 1], [1, 1], [1, 1], [1, 1], 2,
                             2, [4] * 4, mcapa=1)
    c = PD[1][2]
    assert cfl == 0.01 / 0.1 / 0.25 * c  # the left-going wave enters the small cell


def test_transpose_symmetry():
    rng = np.random.default_rng(8)
    mx, my = 17, 22
    q = random_state(2, mx, my, rng)
    aux = kappa(mx, my, rng)
    a, ca, _ = ref.step_aux(2, PD[2], q, aux, 0.03, 0.04, 0.001, [3, 1], [1, 3], [1, 1], [1, 1],
                            2, 2, [4] * 4, mcapa=1)
    qt = np.asfortranarray(q.transpose(0, 2, 1)[[0, 2, 1]])
    at = np.asfortranarray(aux.transpose(0, 2, 1))
    b, cb, _ = ref.step_aux(2, PD[2], qt, at, 0.04, 0.03, 0.001, [1, 3], [3, 1], [1, 1], [1, 1],
                            2, 2, [4] * 4, mcapa=1)
    assert rel_l1(b.transpose(0, 2, 1)[[0, 2, 1]], a) <= 1e-15
    assert ca == cb


def test_lake_at_rest_on_a_nonuniform_grid():
    rng = np.random.default_rng(3)
    mx, my = 19, 23
    b = -(rng.integers(0, 8, size=(mx, my)) / 8.0)
    q = np.zeros((3, mx, my), order="F")
    q[0] = 2.0 - b
    aux = np.empty((2, mx, my), order="F")
    aux[0] = b
    aux[1] = kappa(mx, my, rng)[0]
    out, cfl, rc = ref.step_aux(5, [1.0], q, aux, 0.1, 0.1, 0.01, [3, 3], [3, 3], [1, 1], [1, 1],
                                2, 2, [4] * 3, mcapa=2)
    assert rc == 0
    assert np.array_equal(out, q)


def test_vc_acoustics_with_capacity_in_a_constant_medium():
    """A constant medium makes vc_acoustics constant-coefficient acoustics
    bit for bit, with a capacity too."""
    rng = np.random.default_rng(5)
    mx, my = 26, 20
    q = random_state(4, mx, my, rng)
    rho, bulk = 1.7, 5.3
    c = math.sqrt(bulk / rho)
    k = kappa(mx, my, rng)[0]
    aux = np.empty((3, mx, my), order="F")
    aux[0], aux[1], aux[2] = rho, c, k
    a, ca, ra = ref.step_aux(4, [], q, aux, 0.03, 0.03, 0.001, [3, 1], [1, 3], [3, 1], [1, 3],
                             2, 2, [4] * 2, mcapa=3)
    b, cb, rb = ref.step_aux(1, [rho, bulk, c, rho * c], q, np.asfortranarray(k[None]), 0.03,
                             0.03, 0.001, [3, 1], [1, 3], [3, 1], [1, 3], 2, 2, [4] * 2, mcapa=1)
    assert ra == rb == 0
    assert np.array_equal(a, b)
    assert ca == cb


def test_bad_capacity_index_is_refused():
    q = random_state(1, 8, 8, np.random.default_rng(0))
    with pytest.raises(ValueError):
        ref.step_aux(1, PD[1], q, np.ones((1, 8, 8)), 0.1, 0.1, 0.01, [1, 1], [1, 1], [1, 1],
                     [1, 1], mcapa=2)
