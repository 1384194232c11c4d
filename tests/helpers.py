"""Shared builders for the tests: random physical states per solver."""
import numpy as np

RP_ACOUSTICS, RP_SHALLOW, RP_EULER = 1, 2, 3
SHAPES = {RP_ACOUSTICS: (3, 2), RP_SHALLOW: (3, 3), RP_EULER: (4, 4)}
PD = {RP_ACOUSTICS: [1.0, 4.0, 2.0, 2.0], RP_SHALLOW: [1.0], RP_EULER: [1.4, 1.0]}


def random_state(rp, mx, my, rng):
    m = SHAPES[rp][0]
    q = np.empty((m, mx, my), order="F")
    if rp == RP_ACOUSTICS:
        q[:] = rng.normal(size=(m, mx, my))
    elif rp == RP_SHALLOW:
        q[0] = 1.0 + rng.random((mx, my))
        q[1] = 0.8 * rng.normal(size=(mx, my))
        q[2] = 0.8 * rng.normal(size=(mx, my))
    else:
        rho = 0.3 + rng.random((mx, my))
        u = 0.5 * rng.normal(size=(mx, my))
        v = 0.5 * rng.normal(size=(mx, my))
        p = 0.3 + rng.random((mx, my))
        q[0] = rho
        q[1] = rho * u
        q[2] = rho * v
        q[3] = p / 0.4 + 0.5 * rho * (u * u + v * v)
    return q


def rel_l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())
