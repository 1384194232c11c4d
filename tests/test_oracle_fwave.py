"""Known answers for the f-wave shallow-water solver over bathymetry in the
oracle (rpn2_shallow_bathymetry_fwave, aux = (b,) per cell).

The f-waves sum to the flux difference plus the bathymetry source; the
fluctuations split them by the sign of their speeds; a lake at rest stays at
rest (bit for bit when every operation is exact, to round-off otherwise);
over a flat bottom the first-order step equals the Roe solver's (whose
waves times speeds are the f-waves) to round-off; mass is conserved with
wall boundaries; the step commutes with the x/y transpose."""
import math

import numpy as np
import pytest

from oracle import ref
from tests.helpers import PD, random_bathymetry, random_state, rel_l1

FW, SW = 5, 2


def flux(q, ixy, g):
    h, hu, hv = q
    un = (hu, hv)[ixy - 1]
    f = np.empty(3)
    f[0] = un
    f[ixy] = un * un / h + 0.5 * g * h * h
    f[3 - ixy] = un * (hv if ixy == 1 else hu) / h
    return f


@pytest.mark.parametrize("ixy", [1, 2])
@pytest.mark.parametrize("seed", range(4))
def test_fwaves_sum_to_flux_difference_plus_source(ixy, seed):
    rng = np.random.default_rng(seed)
    g = 9.81
    ql = np.array([1.0 + rng.random(), rng.normal(), rng.normal()])
    qr = np.array([1.0 + rng.random(), rng.normal(), rng.normal()])
    al, ar = np.array([-rng.random()]), np.array([-rng.random()])
    Z, s, am, ap, rc = ref.rpn2_aux(FW, [g], ixy, ql, qr, al, ar)
    assert rc == 0
    hbar = 0.5 * (ql[0] + qr[0])
    delta = flux(qr, ixy, g) - flux(ql, ixy, g)
    delta[ixy] += g * hbar * (ar[0] - al[0])
    assert np.allclose(Z.sum(axis=0), delta, rtol=1e-13, atol=1e-13)
    # Roe speeds, the shear f-wave carries only the transverse momentum
    sl, sr = math.sqrt(ql[0]), math.sqrt(qr[0])
    ubar = (ql[ixy] / sl + qr[ixy] / sr) / (sl + sr)
    c = math.sqrt(g * hbar)
    assert np.allclose(s, [ubar - c, ubar, ubar + c], rtol=1e-14)
    assert Z[1][0] == 0.0 and Z[1][ixy] == 0.0
    neg, pos = Z[s < 0].sum(axis=0), Z[s > 0].sum(axis=0)
    assert np.allclose(am, neg, rtol=1e-15, atol=0) and np.allclose(ap, pos, rtol=1e-15, atol=0)


def test_nonpositive_depth_is_nonphysical():
    Z, s, am, ap, rc = ref.rpn2_aux(FW, [1.0], 1, np.array([0.0, 0, 0]), np.array([1.0, 0, 0]),
                                    np.zeros(1), np.zeros(1))
    assert rc == 2


def lake(mx, my, rng):
    # dyadic depths and bottoms: with g = 1 every operation of the solver is
    # exact on these values
    b = -(rng.integers(0, 8, size=(mx, my)) / 8.0)
    q = np.zeros((3, mx, my), order="F")
    q[0] = 2.0 - b
    aux = np.asfortranarray(b[None])
    return q, aux


@pytest.mark.parametrize("bc", [1, 3])
@pytest.mark.parametrize("order,tw,lim", [(2, 2, 4), (2, 1, 2), (1, 0, 0)])
def test_lake_at_rest_is_exact(bc, order, tw, lim):
    rng = np.random.default_rng(3)
    q, aux = lake(19, 23, rng)
    out, cfl, rc = ref.step_aux(FW, [1.0], q, aux, 0.1, 0.1, 0.01, [bc, bc], [bc, bc], [1, 1],
                                [1, 1], order, tw, [lim] * 3)
    assert rc == 0
    assert np.array_equal(out, q)
    assert cfl > 0.0


def test_lake_at_rest_to_roundoff():
    rng = np.random.default_rng(4)
    mx, my = 31, 27
    aux = random_bathymetry(mx, my, rng)
    q = np.zeros((3, mx, my), order="F")
    q[0] = 1.5 - aux[0]
    out, cfl, rc = ref.step_aux(FW, [9.81], q, aux, 0.02, 0.02, 0.001, [3, 3], [3, 3], [1, 1],
                                [1, 1], 2, 2, [4] * 3)
    assert rc == 0
    assert np.abs(out[0] - q[0]).max() <= 1e-13
    assert np.abs(out[1:]).max() <= 1e-12


@pytest.mark.parametrize("tw", [0, 1, 2])
def test_flat_bottom_first_order_equals_roe(tw):
    rng = np.random.default_rng(10 + tw)
    mx, my = 24, 21
    q = random_state(FW, mx, my, rng)
    aux = np.full((1, mx, my), -0.3, order="F")
    a, ca, ra = ref.step_aux(FW, [9.81], q, aux, 0.05, 0.04, 0.002, [1, 3], [3, 1], [1, 1],
                             [1, 1], 1, tw, [0] * 3)
    b, cb, rb = ref.step(SW, [9.81], q, 0.05, 0.04, 0.002, [1, 3], [3, 1], 1, tw, [0] * 3)
    assert ra == rb == 0
    assert rel_l1(a, b) <= 1e-14
    assert math.isclose(ca, cb, rel_tol=1e-14)


def test_mass_conserved_with_walls():
    rng = np.random.default_rng(6)
    mx, my = 30, 26
    q = random_state(FW, mx, my, rng)
    aux = random_bathymetry(mx, my, rng)
    # the bottom mirrored at the walls too, so that the limited waves at a
    # wall are mirror images and its correction flux carries no mass
    out, cfl, rc = ref.step_aux(FW, PD[FW], q, aux, 0.03, 0.03, 0.001, [3, 3], [3, 3], [3, 3],
                                [3, 3], 2, 2, [4] * 3)
    assert rc == 0
    assert math.isclose(out[0].sum(), q[0].sum(), rel_tol=1e-14)


def test_transpose_symmetry():
    rng = np.random.default_rng(8)
    mx, my = 17, 22
    q = random_state(FW, mx, my, rng)
    aux = random_bathymetry(mx, my, rng)
    a, ca, _ = ref.step_aux(FW, PD[FW], q, aux, 0.03, 0.04, 0.001, [3, 1], [1, 3], [1, 1],
                            [1, 1], 2, 2, [4] * 3)
    qt = np.asfortranarray(q.transpose(0, 2, 1)[[0, 2, 1]])
    at = np.asfortranarray(aux.transpose(0, 2, 1))
    b, cb, _ = ref.step_aux(FW, PD[FW], qt, at, 0.04, 0.03, 0.001, [1, 3], [3, 1], [1, 1],
                            [1, 1], 2, 2, [4] * 3)
    bt = b.transpose(0, 2, 1)[[0, 2, 1]]
    assert rel_l1(bt, a) <= 1e-14
    assert math.isclose(ca, cb, rel_tol=1e-14)
