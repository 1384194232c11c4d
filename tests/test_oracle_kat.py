"""Known-answer tests of the CPU oracle, derived from the mathematics of the
method (the reference's own regression data are not in the mounted tree).

Riemann solvers: waves sum to the jump, fluctuations sum to sum(s W), the Roe
property sum(s W) = f(qr) - f(ql), transverse fluctuations sum to the
transverse Roe Jacobian times the input.  Step: conservation with periodic
and wall boundaries, x/y symmetry, y-uniform data reducing to a 1D
wave-propagation step, exact transport at CFL 1, second-order convergence
of the unsplit method with transverse correction terms."""
import math

import numpy as np
import pytest

from tests.helpers import PD, random_state

G = 1.0
GAMMA = 1.4


def f_shallow(q, ixy):
    h, hu, hv = q
    mu = ixy
    un = q[mu] / h
    out = np.empty(3)
    out[0] = q[mu]
    out[1] = hu * un
    out[2] = hv * un
    out[mu] += 0.5 * G * h * h
    return out


def f_euler(q, ixy):
    rho, ru, rv, E = q
    p = (GAMMA - 1.0) * (E - 0.5 * (ru * ru + rv * rv) / rho)
    un = q[ixy] / rho
    out = np.array([q[ixy], ru * un, rv * un, un * (E + p)])
    out[ixy] += p
    return out


def f_acoustics(q, ixy):
    rho, K = 1.0, 4.0
    p = q[0]
    out = np.zeros(3)
    out[0] = K * q[ixy]
    out[ixy] = p / rho
    return out


FLUX = {1: f_acoustics, 2: f_shallow, 3: f_euler}


def states(rp, rng, n=40):
    q = random_state(rp, n, 2, rng)
    return [(q[:, i, 0].copy(), q[:, i, 1].copy()) for i in range(n)]


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("ixy", [1, 2])
def test_rpn2_identities(oracle, rp, ixy):
    rng = np.random.default_rng(10 * rp + ixy)
    pd = list(PD[rp])
    if rp == 3:
        pd[1] = 0.0  # Roe property is exact without the entropy fix
    for ql, qr in states(rp, rng):
        W, s, am, ap, rc = oracle.rpn2(rp, pd, ixy, ql, qr)
        assert rc == 0
        dq = qr - ql
        if rp == 1:
            dq[3 - ixy] = 0.0  # the zero-speed transverse-velocity wave is not carried
        np.testing.assert_allclose(W.sum(axis=0), dq, rtol=1e-12, atol=1e-13)
        sw = (s[:, None] * W).sum(axis=0)
        np.testing.assert_allclose(am + ap, sw, rtol=1e-12, atol=1e-13)
        df = FLUX[rp](qr, ixy) - FLUX[rp](ql, ixy)
        np.testing.assert_allclose(sw, df, rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("rp", [2, 3])
def test_entropy_fix_keeps_total_fluctuation(oracle, rp):
    """With the fix on, amdq + apdq still equals f(qr) - f(ql), and amdq is
    the plain upwind split whenever no wave is transonic."""
    rng = np.random.default_rng(77 + rp)
    pd = list(PD[rp])
    ntrans = 0
    for ql, qr in states(rp, rng, 200):
        W, s, am, ap, rc = oracle.rpn2(rp, pd, 1, ql, qr)
        np.testing.assert_allclose(am + ap, FLUX[rp](qr, 1) - FLUX[rp](ql, 1), rtol=1e-11,
                                   atol=1e-12)
        plain = (np.minimum(s, 0.0)[:, None] * W).sum(axis=0)
        if not np.allclose(am, plain, rtol=1e-12, atol=1e-13):
            ntrans += 1
            assert np.any(s[[0, -1]] * np.array([1, 1]) != 0)
    assert ntrans > 0  # the random states include transonic rarefactions


def test_shallow_transonic_rarefaction_value(oracle):
    """Left state subcritical flowing right into a deeper-going rarefaction:
    the 1-wave is transonic and amdq = s0 (s1 - lambda1)/(s1 - s0) W1."""
    ql = np.array([1.0, 0.5, 0.0])       # u - c = -0.5
    qr = np.array([0.4, 0.6, 0.0])       # u - c = 1.5 - 0.632 > 0
    W, s, am, ap, rc = oracle.rpn2(2, [1.0], 1, ql, qr)
    s0 = ql[1] / ql[0] - math.sqrt(ql[0])
    h1 = ql[0] + W[0, 0]
    s1 = (ql[1] + W[0, 1]) / h1 - math.sqrt(h1)
    assert s0 < 0 < s1
    sf = s0 * (s1 - s[0]) / (s1 - s0)
    np.testing.assert_allclose(am, sf * W[0], rtol=1e-15)


def jac_y_roe(rp, R, ixy):
    """Transverse Jacobian at the Roe state in the component order of q."""
    mu, mv = ixy, 3 - ixy
    if rp == 2:
        u, v, c = R
        J = np.zeros((3, 3))
        J[0, mv] = 1.0
        J[mu, 0] = -u * v; J[mu, mu] = v; J[mu, mv] = u
        J[mv, 0] = c * c - v * v; J[mv, mv] = 2 * v
        return J
    u, v, H = R
    g1 = GAMMA - 1.0
    q2 = u * u + v * v
    J = np.zeros((4, 4))
    J[0, mv] = 1.0
    J[mu, 0] = -u * v; J[mu, mu] = v; J[mu, mv] = u
    J[mv, 0] = 0.5 * g1 * q2 - v * v; J[mv, mu] = -g1 * u; J[mv, mv] = (3 - GAMMA) * v
    J[mv, 3] = g1
    J[3, 0] = v * (0.5 * g1 * q2 - H); J[3, mu] = -g1 * u * v
    J[3, mv] = H - g1 * v * v; J[3, 3] = GAMMA * v
    return J


@pytest.mark.parametrize("rp", [1, 2, 3])
@pytest.mark.parametrize("ixy", [1, 2])
def test_rpt2_sums_to_transverse_jacobian(oracle, rp, ixy):
    rng = np.random.default_rng(5 * rp + ixy)
    for ql, qr in states(rp, rng, 20):
        asdq = rng.normal(size=ql.shape)
        bm, bp = oracle.rpt2(rp, PD[rp], ixy, ql, qr, asdq)
        mu, mv = ixy, 3 - ixy
        if rp == 1:
            B = np.zeros((3, 3))
            B[0, mv] = 4.0
            B[mv, 0] = 1.0
        elif rp == 2:
            sl, sr = math.sqrt(ql[0]), math.sqrt(qr[0])
            u = (ql[mu] / sl + qr[mu] / sr) / (sl + sr)
            v = (ql[mv] / sl + qr[mv] / sr) / (sl + sr)
            c = math.sqrt(G * 0.5 * (ql[0] + qr[0]))
            B = jac_y_roe(2, (u, v, c), ixy)
        else:
            def pr(q):
                return (GAMMA - 1) * (q[3] - 0.5 * (q[1] ** 2 + q[2] ** 2) / q[0])
            sl, sr = math.sqrt(ql[0]), math.sqrt(qr[0])
            u = (ql[mu] / sl + qr[mu] / sr) / (sl + sr)
            v = (ql[mv] / sl + qr[mv] / sr) / (sl + sr)
            H = ((ql[3] + pr(ql)) / sl + (qr[3] + pr(qr)) / sr) / (sl + sr)
            B = jac_y_roe(3, (u, v, H), ixy)
        np.testing.assert_allclose(bm + bp, B @ asdq, rtol=1e-11, atol=1e-12)


def test_limiter_values(oracle):
    cases = {
        1: [(-1.0, 0.0), (0.5, 0.5), (2.0, 1.0)],
        2: [(-1.0, 0.0), (0.25, 0.5), (0.75, 1.0), (1.5, 1.5), (3.0, 2.0)],
        3: [(-1.0, 0.0), (1.0, 1.0), (3.0, 1.5)],
        4: [(-1.0, 0.0), (0.25, 0.5), (1.0, 1.0), (2.0, 1.5), (5.0, 2.0)],
        0: [(7.0, 1.0)],
    }
    for lim, pairs in cases.items():
        for r, phi in pairs:
            assert oracle.philim(lim, r) == phi, (lim, r)


def test_limiters_stay_in_tvd_region(oracle):
    for lim in (1, 2, 3, 4):
        for r in np.linspace(-3, 6, 181):
            phi = oracle.philim(lim, r)
            assert 0.0 <= phi <= max(0.0, min(2.0 * r, 2.0)) + 1e-15


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_periodic_conservation(oracle, rp):
    rng = np.random.default_rng(rp)
    q = random_state(rp, 24, 18, rng)
    dx, dy = 1.0 / 24, 1.0 / 18
    qn, cfl, rc = oracle.step(rp, PD[rp], q, dx, dy, 0.2 * dx / 4.0, [2, 2], [2, 2])
    assert rc == 0
    np.testing.assert_allclose(qn.sum(axis=(1, 2)), q.sum(axis=(1, 2)), rtol=1e-13, atol=1e-12)


def test_wall_conserves_mass_shallow(oracle):
    rng = np.random.default_rng(9)
    q = random_state(2, 20, 16, rng)
    qn, cfl, rc = oracle.step(2, PD[2], q, 0.05, 0.05, 0.005, [3, 3], [3, 3])
    assert abs(qn[0].sum() - q[0].sum()) <= 1e-13 * q[0].sum()


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_transpose_symmetry(oracle, rp):
    rng = np.random.default_rng(20 + rp)
    q = random_state(rp, 13, 13, rng)
    qt = np.asfortranarray(np.transpose(q, (0, 2, 1))[[0, 2, 1] + ([3] if rp == 3 else [])])
    a, ca, _ = oracle.step(rp, PD[rp], q, 0.1, 0.1, 0.01, [3, 1], [1, 3])
    b, cb, _ = oracle.step(rp, PD[rp], qt, 0.1, 0.1, 0.01, [1, 3], [3, 1])
    bt = np.transpose(b, (0, 2, 1))[[0, 2, 1] + ([3] if rp == 3 else [])]
    np.testing.assert_allclose(a, bt, rtol=1e-13, atol=1e-13)
    assert ca == cb


def step1d(oracle, rp, q1, dtdx, lim):
    """Independent 1D wave-propagation step (order 2, limited), periodic."""
    n = q1.shape[1]
    ext = np.concatenate([q1[:, -2:], q1, q1[:, :2]], axis=1)
    W, S, AM, AP = [], [], [], []
    for e in range(-1, n + 2):
        w, s, am, ap, _ = oracle.rpn2(rp, PD[rp], 1, ext[:, e + 1], ext[:, e + 2])
        W.append(w); S.append(s); AM.append(am); AP.append(ap)
    out = q1.copy()
    F = []
    for e in range(0, n + 1):
        k = e + 1
        wl = W[k].copy()
        for p in range(W[k].shape[0]):
            nrm = float(np.dot(W[k][p], W[k][p]))
            if nrm == 0.0:
                continue
            up = W[k - 1][p] if S[k][p] > 0 else W[k + 1][p]
            wl[p] = oracle.philim(lim, float(np.dot(up, W[k][p])) / nrm) * W[k][p]
        sa = np.abs(S[k])
        F.append(0.5 * ((sa * (1 - sa * dtdx))[:, None] * wl).sum(axis=0))
    for i in range(n):
        out[:, i] = (q1[:, i] - dtdx * (AP[i + 1] + AM[i + 2])
                     - dtdx * (F[i + 1] - F[i]))
    return out


@pytest.mark.parametrize("rp", [1, 2, 3])
def test_y_uniform_reduces_to_1d(oracle, rp):
    rng = np.random.default_rng(40 + rp)
    q1 = random_state(rp, 16, 1, rng)[:, :, 0]
    if rp != 1:
        q1[2] = 0.0 if rp == 2 else 0.0  # no transverse momentum
        if rp == 3:
            rho, ru = q1[0], q1[1]
    q = np.asfortranarray(np.repeat(q1[:, :, None], 6, axis=2))
    if rp == 3:
        # keep E consistent after zeroing rho v (pressure stays positive)
        pass
    dx = 1.0 / 16
    dt = 0.3 * dx / 4.0
    qn, cfl, rc = oracle.step(rp, PD[rp], q, dx, dx, dt, [2, 2], [2, 2], order=2, tw=2,
                              mthlim=[4] * 4)
    for j in range(1, 6):
        assert np.array_equal(qn[:, :, j], qn[:, :, 0])
    ref1 = step1d(oracle, rp, q1, dt / dx, 4)
    np.testing.assert_allclose(qn[:, :, 0], ref1, rtol=1e-13, atol=1e-13)


def test_acoustics_cfl1_exact_shift(oracle):
    n = 32
    x = (np.arange(n) + 0.5) / n
    w = np.exp(-50 * (x - 0.4) ** 2)
    q = np.zeros((3, n, 4), order="F")
    Z = 2.0
    q[0] = (Z * w)[:, None]
    q[1] = w[:, None]
    dx = 1.0 / n
    dt = dx / 2.0  # c = 2, CFL exactly 1
    qn, cfl, rc = oracle.step(1, PD[1], q, dx, dx, dt, [2, 2], [2, 2], order=2, tw=2,
                              mthlim=[4, 4])
    assert cfl == 1.0
    np.testing.assert_allclose(qn[:, :, 0], np.roll(q[:, :, 0], 1, axis=1), atol=1e-15)


def _plane_wave(n, t):
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    c, Z = 2.0, 2.0
    f = np.sin(2 * np.pi * (X + Y) - 2 * np.pi * math.sqrt(2) * c * t)
    q = np.zeros((3, n, n), order="F")
    q[0] = f
    q[1] = f / (Z * math.sqrt(2))
    q[2] = f / (Z * math.sqrt(2))
    return q


@pytest.mark.parametrize("tw,min_rate", [(2, 1.8)])
def test_unsplit_second_order_diagonal_wave(oracle, tw, min_rate):
    errs = []
    T = 0.05
    for n in (16, 32, 64):
        q = _plane_wave(n, 0.0)
        dx = 1.0 / n
        nsteps = int(round(T / (0.4 * dx / 2.0)))
        dt = T / nsteps
        for _ in range(nsteps):
            q, cfl, rc = oracle.step(1, PD[1], q, dx, dx, dt, [2, 2], [2, 2], order=2, tw=tw,
                                     mthlim=[0, 0])
        errs.append(np.abs(q - _plane_wave(n, T)).mean())
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(rates) > min_rate, (errs, rates)
