"""Known answers for variable-coefficient acoustics in the oracle
(rpn2/rpt2_vc_acoustics, aux = (rho, c) per cell).

Constant coefficients reproduce constant-coefficient acoustics bit for bit
(single steps, every boundary mix, limiter, order and transverse option);
the interface Riemann problem gives waves that sum to the jump, speeds -c_l
and +c_r, and the classical transmission and reflection coefficients; the
transverse split equals the constant-coefficient split for a uniform
column and transmits (not reflects) into a matched medium."""
import math

import numpy as np
import pytest

from oracle import ref
from tests.helpers import PD, random_medium, random_state

VC, AC = 4, 1


def constant_medium(mx, my, rho, bulk):
    c = math.sqrt(bulk / rho)
    aux = np.empty((2, mx, my), order="F")
    aux[0], aux[1] = rho, c
    return aux, [rho, bulk, c, rho * c]


@pytest.mark.parametrize("bcl,bcu", [([1, 1], [1, 1]), ([3, 3], [3, 3]), ([2, 2], [2, 2]),
                                     ([3, 1], [1, 3])])
@pytest.mark.parametrize("order,tw,lim", [(2, 2, 4), (2, 1, 1), (2, 0, 2), (1, 0, 0), (1, 2, 3)])
def test_constant_medium_equals_acoustics(bcl, bcu, order, tw, lim):
    rng = np.random.default_rng(11 * order + tw + lim)
    q = random_state(AC, 23, 17, rng)
    aux, pd = constant_medium(23, 17, 1.7, 5.3)
    a, ca, ra = ref.step_aux(VC, [], q, aux, 0.04, 0.05, 0.003, bcl, bcu, bcl, bcu, order, tw,
                             [lim] * 4)
    b, cb, rb = ref.step(AC, pd, q, 0.04, 0.05, 0.003, bcl, bcu, order, tw, [lim] * 4)
    assert ra == rb == 0
    assert np.array_equal(a, b)
    assert ca == cb


@pytest.mark.parametrize("ixy", [1, 2])
def test_interface_riemann_problem(ixy):
    rng = np.random.default_rng(ixy)
    ql, qr = rng.normal(size=3), rng.normal(size=3)
    al, ar = np.array([1.3, 0.7]), np.array([2.9, 1.9])
    W, s, am, ap, rc = ref.rpn2_aux(VC, [], ixy, ql, qr, al, ar)
    assert rc == 0
    assert np.allclose(W.sum(axis=0)[[0, ixy]], (qr - ql)[[0, ixy]], rtol=1e-14, atol=1e-14)
    assert np.all(W[:, 3 - ixy] == 0.0)
    assert s[0] == -al[1] and s[1] == ar[1]
    assert np.array_equal(am, s[0] * W[0]) and np.array_equal(ap, s[1] * W[1])
    # an incident right-going wave (p, u) = (Zl, 1) meeting the interface at rest
    zl, zr = al[0] * al[1], ar[0] * ar[1]
    q_in = np.zeros(3)
    q_in[0], q_in[ixy] = zl, 1.0
    W, s, am, ap, _ = ref.rpn2_aux(VC, [], ixy, q_in, np.zeros(3), al, ar)
    # the state between the waves, q_in + W1: transmitted pressure T*zl, with
    # T = 2 zr / (zl + zr); reflected pressure wave R*zl, R = (zr - zl)/(zl + zr)
    mid = q_in + W[0]
    assert math.isclose(mid[0], 2.0 * zr / (zl + zr) * zl, rel_tol=1e-14)
    assert math.isclose(W[0][0], (zr - zl) / (zl + zr) * zl, rel_tol=1e-14)


@pytest.mark.parametrize("ixy", [1, 2])
def test_transverse_split(ixy):
    rng = np.random.default_rng(5 + ixy)
    asdq = rng.normal(size=3)
    rho, bulk = 1.6, 3.1
    c = math.sqrt(bulk / rho)
    a = np.array([rho, c])
    bm, bp = ref.rpt2_aux(VC, [], ixy, a, a, a, asdq)
    bm0, bp0 = ref.rpt2(AC, [rho, bulk, c, rho * c], ixy, None, None, asdq)
    assert np.array_equal(bm, bm0) and np.array_equal(bp, bp0)
    # a matched medium below (same impedance, other speed): the down-going
    # part is transmitted with the speed of the cell below
    am = np.array([rho * c / 0.5, 0.5])
    bm1, _ = ref.rpt2_aux(VC, [], ixy, am, a, a, asdq)
    assert np.allclose(bm1, bm0 * 0.5 / c, rtol=1e-14)
    assert bm1[ixy] == 0.0 and bp[ixy] == 0.0


def test_layered_medium_wall_run_stays_bounded():
    """A 40x30 layered medium with walls for 60 steps: finite, Courant
    number from the fastest layer, energy not growing."""
    rng = np.random.default_rng(2)
    aux = random_medium(40, 30, rng)
    q = np.zeros((3, 40, 30), order="F")
    X, Y = np.meshgrid(np.arange(40), np.arange(30), indexing="ij")
    q[0] = np.exp(-0.05 * ((X - 20.0) ** 2 + (Y - 15.0) ** 2))
    dx = dy = 1.0 / 40
    cmax = aux[1].max()
    dt = 0.8 * dx / cmax
    rho, c = aux
    energy = lambda q: float((0.5 * q[0] ** 2 / (rho * c * c) + 0.5 * rho * (q[1] ** 2 + q[2] ** 2)).sum())  # noqa: E731
    e0 = energy(q)
    for _ in range(60):
        q, cfl, rc = ref.step_aux(VC, [], q, aux, dx, dy, dt, [3, 3], [3, 3], [3, 3], [3, 3])
        assert rc == 0 and cfl <= 0.8 * (1 + 1e-12)
    assert np.all(np.isfinite(q))
    assert energy(q) <= e0 * (1 + 1e-12)
