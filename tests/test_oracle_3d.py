"""Known answers for the unsplit 3D step in the oracle (classic3_ref.c).

Constant-velocity advection pins the transverse algebra: with order 1 and
transverse_waves 11 the step is the corner transport upwind scheme, i.e.
trilinear upwind interpolation, for every sign pattern of the velocity; with
transverse_waves 0 it is donor cell.  Acoustics on data that do not vary in
z reproduces the 2D step (the z-transverse and corner terms cancel); the
step conserves every component with periodic boundaries, keeps a constant
state bit for bit, commutes with a cyclic permutation of the axes, and
reports c dt / min(dx, dy, dz) as its Courant number.  The 3D Euler Roe
solver's waves sum to the jump and their speed-weighted sum to the flux
difference (the Roe property); at first order, data that do not vary in z
reproduce the 2D Euler step without entropy fix; it conserves, keeps
constant states and commutes with the cyclic axis permutation."""
import math

import numpy as np
import pytest

from oracle import ref
from tests.helpers import rel_l1

AC3, EU3, ADV3 = ref.RP3_ACOUSTICS, ref.RP3_EULER, ref.RP3_ADVECTION
PD3 = [1.0, 4.0, 2.0, 2.0]  # rho, bulk, c, Z


def random3(m, shape, rng):
    return np.asfortranarray(rng.normal(size=(m,) + shape))


def trilinear(q, nu):
    """Corner transport upwind: each cell takes the trilinear interpolation
    of the upwind 2x2x2 block at its departure point (periodic)."""
    out = np.zeros_like(q)
    ax = []
    for d, n in enumerate(nu):
        s = 1 if n > 0 else -1
        ax.append([(0, 1.0 - abs(n)), (s, abs(n))])
    for sx, wx in ax[0]:
        for sy, wy in ax[1]:
            for sz, wz in ax[2]:
                out += wx * wy * wz * np.roll(q, (sx, sy, sz), axis=(1, 2, 3))
    return out


@pytest.mark.parametrize("vel", [(1.0, 0.7, 0.4), (-0.8, 0.5, -0.3), (0.6, -0.9, 0.2),
                                 (-0.5, -0.4, -0.7)])
def test_advection_is_corner_transport_upwind(vel):
    rng = np.random.default_rng(1)
    shape = (9, 8, 7)
    q = random3(1, shape, rng)
    dt = 0.08
    dx, dy, dz = 0.1, 0.12, 0.09
    out, cfl = ref.step3(ADV3, list(vel), q, dx, dy, dz, dt, [2] * 3, [2] * 3, 1, 11, [0])
    nu = (vel[0] * dt / dx, vel[1] * dt / dy, vel[2] * dt / dz)
    assert np.allclose(out, trilinear(q, nu), rtol=0, atol=1e-14)
    assert math.isclose(cfl, max(abs(n) for n in nu), rel_tol=1e-15)


def test_advection_donor_cell():
    rng = np.random.default_rng(2)
    q = random3(1, (8, 9, 10), rng)
    vel, dt, h = (0.9, -0.6, 0.3), 0.05, 0.1
    out, _ = ref.step3(ADV3, list(vel), q, h, h, h, dt, [2] * 3, [2] * 3, 1, 0, [0])
    expect = q.copy()
    for d, v in enumerate(vel):
        nu = v * dt / h
        up = np.roll(q, 1 if v > 0 else -1, axis=d + 1)
        expect -= abs(nu) * (q - up)
    assert np.allclose(out, expect, rtol=0, atol=1e-14)


@pytest.mark.parametrize("order,tw,tw2", [(2, 22, 2), (2, 20, 2), (2, 11, 1), (1, 10, 1),
                                          (2, 0, 0)])
def test_z_uniform_acoustics_is_the_2d_step(order, tw, tw2):
    rng = np.random.default_rng(3 + tw)
    mx, my, mz = 13, 11, 5
    q2 = rng.normal(size=(3, mx, my))
    q3 = np.zeros((4, mx, my, mz), order="F")
    q3[:3] = q2[..., None]
    dx, dy, dz, dt = 0.1, 0.12, 0.07, 0.01
    bcl, bcu = [1, 3], [3, 1]
    out3, cfl3 = ref.step3(AC3, PD3, q3, dx, dy, dz, dt, bcl + [2], bcu + [2], order, tw,
                           [4, 4])
    out2, cfl2, rc = ref.step(1, PD3, np.asfortranarray(q2), dx, dy, dt, bcl, bcu, order, tw2,
                              [4, 4])
    for l in range(mz):
        assert rel_l1(out3[:3, :, :, l], out2) <= 1e-14
    assert np.abs(out3[3]).max() <= 1e-14
    assert cfl3 == pytest.approx(PD3[2] * dt / dz, rel=1e-15)


@pytest.mark.parametrize("tw", [22, 11, 20])
def test_conservation_periodic(tw):
    rng = np.random.default_rng(4)
    q = random3(4, (10, 9, 8), rng)
    out, _ = ref.step3(AC3, PD3, q, 0.1, 0.1, 0.1, 0.02, [2] * 3, [2] * 3, 2, tw, [4, 4])
    for k in range(4):
        assert abs(out[k].sum() - q[k].sum()) <= 1e-13 * np.abs(q[k]).sum()


def test_constant_state_preserved():
    q = np.empty((4, 7, 6, 5), order="F")
    q[:] = np.array([0.3, -1.2, 0.5, 2.0])[:, None, None, None]
    out, _ = ref.step3(AC3, PD3, q, 0.1, 0.1, 0.1, 0.02, [1, 2, 1], [1, 2, 1], 2, 22, [4, 4])
    assert np.array_equal(out, q)


def test_cyclic_axis_permutation():
    rng = np.random.default_rng(5)
    q = random3(4, (9, 8, 7), rng)
    dx, dy, dz, dt = 0.1, 0.13, 0.08, 0.012
    a, ca = ref.step3(AC3, PD3, q, dx, dy, dz, dt, [1, 3, 2], [1, 3, 2], 2, 22, [4, 4])
    # new axes (x', y', z') = (y, z, x): velocities (u', v', w') = (v, w, u)
    qp = np.asfortranarray(q.transpose(0, 2, 3, 1)[[0, 2, 3, 1]])
    b, cb = ref.step3(AC3, PD3, qp, dy, dz, dx, dt, [3, 2, 1], [3, 2, 1], 2, 22, [4, 4])
    back = b[[0, 3, 1, 2]].transpose(0, 3, 1, 2)
    assert rel_l1(back, a) <= 1e-14
    assert ca == cb


def test_unsupported_transverse_option():
    q = random3(4, (4, 4, 4), np.random.default_rng(0))
    with pytest.raises(ValueError):
        ref.step3(AC3, PD3, q, 0.1, 0.1, 0.1, 0.01, [1] * 3, [1] * 3, 2, 21, [4, 4])


def euler_state(shape, rng, gamma=1.4):
    rho = 0.5 + rng.random(shape)
    u = 0.5 * rng.normal(size=(3,) + shape)
    p = 0.5 + rng.random(shape)
    q = np.empty((5,) + shape, order="F")
    q[0] = rho
    q[1:4] = rho * u
    q[4] = p / (gamma - 1.0) + 0.5 * rho * (u ** 2).sum(axis=0)
    return q


def euler_flux(q, d, gamma=1.4):
    rho, m = q[0], q[1:4]
    p = (gamma - 1.0) * (q[4] - 0.5 * (m ** 2).sum() / rho)
    un = m[d] / rho
    f = un * q
    f[1 + d] += p
    f[4] += un * p
    return f


@pytest.mark.parametrize("d", [0, 1, 2])
@pytest.mark.parametrize("seed", range(3))
def test_euler_roe_property(d, seed):
    rng = np.random.default_rng(seed)
    ql = euler_state((), rng)
    qr = euler_state((), rng)
    W, s, am, ap, rc = ref.rpn3(EU3, [1.4], d, ql, qr)
    assert rc == 0
    assert np.allclose(W.sum(axis=0), qr - ql, rtol=1e-13, atol=1e-13)
    df = euler_flux(qr, d) - euler_flux(ql, d)
    assert np.allclose(am + ap, df, rtol=1e-12, atol=1e-12)
    assert np.allclose((s[:, None] * W).sum(axis=0), df, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("tw,tw2", [(10, 1), (11, 1), (0, 0)])
def test_euler_z_uniform_first_order_is_the_2d_step(tw, tw2):
    rng = np.random.default_rng(40 + tw)
    mx, my, mz = 13, 11, 4
    q2 = euler_state((mx, my), rng)
    q2[3] = 0.0  # no z momentum
    q2[4] = 1.5 / 0.4 + 0.5 * (q2[1] ** 2 + q2[2] ** 2) / q2[0]
    q3 = np.zeros((5, mx, my, mz), order="F")
    q3[0:3] = q2[0:3, ..., None]
    q3[4] = q2[4, ..., None]
    dx, dy, dz, dt = 0.1, 0.12, 0.07, 0.005
    bcl, bcu = [1, 3], [3, 1]
    out3, cfl3 = ref.step3(EU3, [1.4], q3, dx, dy, dz, dt, bcl + [2], bcu + [2], 1, tw, [0] * 3)
    q24 = np.asfortranarray(q2[[0, 1, 2, 4]])
    out2, cfl2, rc = ref.step(3, [1.4, 0.0], q24, dx, dy, dt, bcl, bcu, 1, tw2, [0] * 4)
    assert rc == 0
    for l in range(mz):
        assert rel_l1(out3[[0, 1, 2, 4], :, :, l], out2) <= 1e-14
    assert np.abs(out3[3]).max() <= 1e-14


def test_euler_conservation_constant_state_and_permutation():
    rng = np.random.default_rng(50)
    q = euler_state((9, 8, 7), rng)
    out, _ = ref.step3(EU3, [1.4], q, 0.1, 0.1, 0.1, 0.004, [2] * 3, [2] * 3, 2, 22, [4] * 3)
    for k in range(5):
        assert abs(out[k].sum() - q[k].sum()) <= 1e-13 * np.abs(q[k]).sum()
    c = np.empty((5, 6, 5, 4), order="F")
    c[:] = euler_state((), rng)[:, None, None, None]
    outc, _ = ref.step3(EU3, [1.4], c, 0.1, 0.1, 0.1, 0.004, [1, 2, 1], [1, 2, 1], 2, 22,
                        [4] * 3)
    assert np.array_equal(outc, c)
    dx, dy, dz, dt = 0.1, 0.13, 0.08, 0.004
    a, ca = ref.step3(EU3, [1.4], q, dx, dy, dz, dt, [1, 3, 2], [1, 3, 2], 2, 22, [4] * 3)
    qp = np.asfortranarray(q.transpose(0, 2, 3, 1)[[0, 2, 3, 1, 4]])
    b, cb = ref.step3(EU3, [1.4], qp, dy, dz, dx, dt, [3, 2, 1], [3, 2, 1], 2, 22, [4] * 3)
    back = b[[0, 3, 1, 2, 4]].transpose(0, 3, 1, 2)
    assert rel_l1(back, a) <= 1e-14
    assert ca == cb


def test_split_step_is_three_one_dimensional_sweeps():
    """The split step equals x, y and z sweeps of the unsplit step without
    transverse terms on data that vary along one axis only (each sweep then
    sees the same 1D problem), and conserves with periodic boundaries."""
    rng = np.random.default_rng(60)
    mx, my, mz = 16, 5, 4
    prof = rng.normal(size=(4, mx))
    q = np.zeros((4, mx, my, mz), order="F")
    q[:] = prof[:, :, None, None]
    q[2:] = 0.0  # no transverse velocity
    d = (0.1, 0.12, 0.09)
    dt = 0.01
    a, ca = ref.step3_split(AC3, PD3, q, *d, dt, [1, 2, 2], [1, 2, 2], 2, [4, 4])
    b, cb = ref.step3(AC3, PD3, q, *d, dt, [1, 2, 2], [1, 2, 2], 2, 0, [4, 4])
    assert rel_l1(a, b) <= 1e-15
    r = random3(4, (9, 8, 7), rng)
    out, _ = ref.step3_split(AC3, PD3, r, 0.1, 0.1, 0.1, 0.02, [2] * 3, [2] * 3, 2, [4, 4])
    for k in range(4):
        assert abs(out[k].sum() - r[k].sum()) <= 1e-13 * np.abs(r[k]).sum()
    e = euler_state((8, 7, 6), rng)
    oute, _ = ref.step3_split(EU3, [1.4], e, 0.1, 0.1, 0.1, 0.004, [2] * 3, [2] * 3, 2, [4] * 3)
    for k in range(5):
        assert abs(oute[k].sum() - e[k].sum()) <= 1e-13 * np.abs(e[k]).sum()


@pytest.mark.parametrize("order,lim", [(2, 4), (2, 1), (1, 0)])
def test_z_uniform_split_is_the_2d_split_step(order, lim):
    """On z-uniform data without z-velocity the z-sweep does nothing and the
    x- and y-sweeps are those of the 2D split step (an independent
    restatement, pinned by the 2D known answers)."""
    rng = np.random.default_rng(70 + lim)
    mx, my, mz = 14, 9, 4
    q2 = rng.normal(size=(3, mx, my))
    q3 = np.zeros((4, mx, my, mz), order="F")
    q3[:3] = q2[..., None]
    dx, dy, dz, dt = 0.1, 0.12, 0.5, 0.01
    bcl, bcu = [1, 3], [3, 2]
    out3, cfl3 = ref.step3_split(AC3, PD3, q3, dx, dy, dz, dt, bcl + [2], bcu + [2], order,
                                 [lim, lim])
    out2, cfl2, rc = ref.step_split(1, PD3, np.asfortranarray(q2), dx, dy, dt, bcl, bcu, order,
                                    [lim, lim])
    for l in range(mz):
        assert rel_l1(out3[:3, :, :, l], out2) <= 1e-15
    assert np.abs(out3[3]).max() == 0.0
    assert cfl3 == pytest.approx(cfl2, rel=1e-15)


def test_euler_z_uniform_first_order_split_is_the_2d_split_step():
    """The split Euler step on z-uniform data without z-momentum, at first
    order, equals the 2D split step of the 4-wave solver without entropy fix
    (without limiting, grouping the entropy and shear waves changes
    nothing); the z-sweep leaves the data as it is."""
    rng = np.random.default_rng(77)
    mx, my, mz = 14, 10, 4
    q2 = euler_state((mx, my), rng)
    q2[3] = 0.0
    q2[4] = 1.5 / 0.4 + 0.5 * (q2[1] ** 2 + q2[2] ** 2) / q2[0]
    q3 = np.zeros((5, mx, my, mz), order="F")
    q3[0:3] = q2[0:3, ..., None]
    q3[4] = q2[4, ..., None]
    dx, dy, dz, dt = 0.1, 0.12, 0.5, 0.004
    bcl, bcu = [1, 3], [3, 1]
    out3, cfl3 = ref.step3_split(EU3, [1.4], q3, dx, dy, dz, dt, bcl + [2], bcu + [2], 1,
                                 [0] * 3)
    q24 = np.asfortranarray(q2[[0, 1, 2, 4]])
    out2, cfl2, rc = ref.step_split(3, [1.4, 0.0], q24, dx, dy, dt, bcl, bcu, 1, [0] * 4)
    assert rc == 0
    for l in range(mz):
        assert rel_l1(out3[[0, 1, 2, 4], :, :, l], out2) <= 1e-14
    assert np.abs(out3[3]).max() <= 1e-14


def _plane_wave3(n, t):
    """A pressure wave along (1, 1, 1) on the periodic unit cube: p =
    sin(2 pi (x + y + z - sqrt(3) c t)), velocity p / Z along the
    direction, exact for constant-coefficient acoustics."""
    x = (np.arange(n) + 0.5) / n
    X, Y, Z3 = np.meshgrid(x, x, x, indexing="ij")
    c, Z = PD3[2], PD3[3]
    f = np.sin(2 * np.pi * (X + Y + Z3) - 2 * np.pi * math.sqrt(3) * c * t)
    q = np.zeros((4, n, n, n), order="F")
    q[0] = f
    q[1] = q[2] = q[3] = f / (Z * math.sqrt(3))
    return q


@pytest.mark.parametrize("tw", [22, 20])
def test_unsplit_second_order_diagonal_wave(tw):
    """Without limiting the unsplit 3D step converges at second order on a
    smooth wave crossing the grid diagonally (the order the transverse and
    corner terms exist for)."""
    errs = []
    T = 0.05
    for n in (16, 32, 64):
        q = _plane_wave3(n, 0.0)
        dx = 1.0 / n
        nsteps = int(round(T / (0.4 * dx / PD3[2])))
        dt = T / nsteps
        for _ in range(nsteps):
            q, _ = ref.step3(AC3, PD3, q, dx, dx, dx, dt, [2] * 3, [2] * 3, 2, tw, [0, 0],
                             nthreads=8)
        errs.append(np.abs(q - _plane_wave3(n, T)).mean())
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(rates) > 1.8, (errs, rates)
