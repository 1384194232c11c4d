"""Shared builders for the tests: random physical states per solver."""
import numpy as np

RP_ACOUSTICS, RP_SHALLOW, RP_EULER, RP_VC_ACOUSTICS, RP_SHALLOW_FWAVE = 1, 2, 3, 4, 5
SHAPES = {RP_ACOUSTICS: (3, 2), RP_SHALLOW: (3, 3), RP_EULER: (4, 4), RP_VC_ACOUSTICS: (3, 2),
          RP_SHALLOW_FWAVE: (3, 3)}
PD = {RP_ACOUSTICS: [1.0, 4.0, 2.0, 2.0], RP_SHALLOW: [1.0], RP_EULER: [1.4, 1.0],
      RP_VC_ACOUSTICS: [], RP_SHALLOW_FWAVE: [9.81]}


def random_state(rp, mx, my, rng):
    m = SHAPES[rp][0]
    q = np.empty((m, mx, my), order="F")
    if rp in (RP_ACOUSTICS, RP_VC_ACOUSTICS):
        q[:] = rng.normal(size=(m, mx, my))
    elif rp in (RP_SHALLOW, RP_SHALLOW_FWAVE):
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


def random_medium(mx, my, rng):
    """aux = (rho, c) of a layered, noisy medium for variable-coefficient
    acoustics: densities in [0.5, 3], sound speeds in [0.5, 2.5]."""
    aux = np.empty((2, mx, my), order="F")
    layer = (np.arange(mx)[:, None] + 2 * np.arange(my)[None, :]) % 7 < 3
    aux[0] = np.where(layer, 2.5, 0.6) + 0.4 * rng.random((mx, my))
    aux[1] = np.where(layer, 0.6, 2.0) + 0.4 * rng.random((mx, my))
    return aux


def random_bathymetry(mx, my, rng, amp=0.5):
    """aux = (b,) for the f-wave shallow-water solver: a smooth bump plus
    noise, below the depths random_state draws (h in [1, 2])."""
    x = (np.arange(mx)[:, None] + 0.5) / mx
    y = (np.arange(my)[None, :] + 0.5) / my
    aux = np.empty((1, mx, my), order="F")
    aux[0] = -1.0 + amp * np.exp(-20.0 * ((x - 0.4) ** 2 + (y - 0.6) ** 2))
    aux[0] += 0.05 * amp * rng.random((mx, my))
    return aux
