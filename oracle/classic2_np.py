"""Second, independent CPU restatement of the classic unsplit 2D step (numpy).

TEST INFRASTRUCTURE ONLY (the checker; never imported by the product path).
PARITY UNPINNED: the reference's Fortran (upstream
pyclaw/src/pyclaw/classic/{step2,flux2,limiter}.f90 and
riemann/src/rpn2_*/rpt2_* .f90, git submodules that are empty in clawpack
5.14.0's umbrella tree, .gitmodules:1-21) cannot be read or built here.

This module vectorises over every slice of a sweep at once instead of looping
over slices like ``classic2_ref.c``; it is written separately so that an
indexing or ordering mistake in one restatement shows up against the other.
Every element sees the same sequence of IEEE operations as in the C oracle,
so the two agree bit for bit (numpy never fuses multiply-adds).

Layout: ``qbc`` has shape ``(m, mx+4, my+4)`` (PyClaw's qbc, num_ghost = 2).
"""
from __future__ import annotations

import numpy as np

RP_ACOUSTICS, RP_SHALLOW, RP_EULER = 1, 2, 3
BC_EXTRAP, BC_PERIODIC, BC_WALL = 1, 2, 3
SHAPES = {RP_ACOUSTICS: (3, 2), RP_SHALLOW: (3, 3), RP_EULER: (4, 4)}


def fill_ghosts(q, bc_lower, bc_upper, g=2):
    """PyClaw _apply_bcs for one process: x boundaries over all rows, then y
    boundaries over all columns (upstream pyclaw/src/pyclaw/solver.py)."""
    m, mx, my = q.shape
    qbc = np.zeros((m, mx + 2 * g, my + 2 * g))
    qbc[:, g:g + mx, g:g + my] = q
    for d, n in ((0, mx), (1, my)):
        a = np.moveaxis(qbc, d + 1, 1)  # view with the swept axis second
        comp = d + 1
        for l in range(g):
            if bc_lower[d] == BC_EXTRAP:
                a[:, l] = a[:, g]
            elif bc_lower[d] == BC_PERIODIC:
                a[:, l] = a[:, l + n]
            else:
                a[:, l] = a[:, 2 * g - 1 - l]
                a[comp, l] = -a[comp, 2 * g - 1 - l]
            if bc_upper[d] == BC_EXTRAP:
                a[:, g + n + l] = a[:, g + n - 1]
            elif bc_upper[d] == BC_PERIODIC:
                a[:, g + n + l] = a[:, g + l]
            else:
                a[:, g + n + l] = a[:, g + n - 1 - l]
                a[comp, g + n + l] = -a[comp, g + n - 1 - l]
    return qbc


# ---------------------------------------------------------------- Riemann solvers
# ql, qr: arrays (..., m); returns wave (..., mw, m), s (..., mw), amdq, apdq (..., m)

def _rpn2_acoustics(pd, ixy, ql, qr):
    cc, zz = pd[2], pd[3]
    mu, mv = ixy, 3 - ixy
    d0 = qr[..., 0] - ql[..., 0]
    d1 = qr[..., mu] - ql[..., mu]
    a1 = (-d0 + zz * d1) / (2.0 * zz)
    a2 = (d0 + zz * d1) / (2.0 * zz)
    sh = ql.shape[:-1]
    wave = np.zeros(sh + (2, 3))
    s = np.empty(sh + (2,))
    wave[..., 0, 0] = -a1 * zz
    wave[..., 0, mu] = a1
    wave[..., 1, 0] = a2 * zz
    wave[..., 1, mu] = a2
    s[..., 0] = -cc
    s[..., 1] = cc
    amdq = s[..., 0, None] * wave[..., 0, :]
    apdq = s[..., 1, None] * wave[..., 1, :]
    return wave, s, amdq, apdq


def _rpn2_shallow(pd, ixy, ql, qr):
    g = pd[0]
    mu, mv = ixy, 3 - ixy
    hl, hr = ql[..., 0], qr[..., 0]
    hsl, hsr = np.sqrt(hl), np.sqrt(hr)
    hsq2 = hsl + hsr
    u = (ql[..., mu] / hsl + qr[..., mu] / hsr) / hsq2
    v = (ql[..., mv] / hsl + qr[..., mv] / hsr) / hsq2
    c = np.sqrt(g * ((hl + hr) * 0.5))
    d0 = hr - hl
    d1 = qr[..., mu] - ql[..., mu]
    d2 = qr[..., mv] - ql[..., mv]
    a1 = ((u + c) * d0 - d1) * (0.5 / c)
    a2 = -v * d0 + d2
    a3 = (-(u - c) * d0 + d1) * (0.5 / c)
    sh = ql.shape[:-1]
    wave = np.zeros(sh + (3, 3))
    s = np.empty(sh + (3,))
    wave[..., 0, 0] = a1
    wave[..., 0, mu] = a1 * (u - c)
    wave[..., 0, mv] = a1 * v
    wave[..., 1, mv] = a2
    wave[..., 2, 0] = a3
    wave[..., 2, mu] = a3 * (u + c)
    wave[..., 2, mv] = a3 * v
    s[..., 0] = u - c
    s[..., 1] = u
    s[..., 2] = u + c
    # Harten-Hyman entropy fix
    s0 = ql[..., mu] / hl - np.sqrt(g * hl)
    h1 = hl + wave[..., 0, 0]
    hu1 = ql[..., mu] + wave[..., 0, mu]
    s1 = hu1 / h1 - np.sqrt(g * h1)
    trans1 = (s0 < 0.0) & (s1 > 0.0)
    sf1 = np.where(trans1, s0 * (s1 - s[..., 0]) / (s1 - s0),
                   np.where(s[..., 0] < 0.0, s[..., 0], 0.0))
    amdq = sf1[..., None] * wave[..., 0, :]
    go2 = s[..., 1] < 0.0
    amdq = np.where(go2[..., None], amdq + s[..., 1, None] * wave[..., 1, :], amdq)
    s03 = qr[..., mu] / hr + np.sqrt(g * hr)
    h3 = hr - wave[..., 2, 0]
    hu3 = qr[..., mu] - wave[..., 2, mu]
    s3 = hu3 / h3 + np.sqrt(g * h3)
    trans3 = (s3 < 0.0) & (s03 > 0.0)
    sf3 = np.where(trans3, s3 * (s03 - s[..., 2]) / (s03 - s3), s[..., 2])
    add3 = go2 & (trans3 | (s[..., 2] < 0.0))
    amdq = np.where(add3[..., None], amdq + sf3[..., None] * wave[..., 2, :], amdq)
    allright = (s0 >= 0.0) & (s[..., 0] > 0.0)
    amdq = np.where(allright[..., None], 0.0, amdq)
    df = np.zeros_like(amdq)
    for p in range(3):
        df = df + s[..., p, None] * wave[..., p, :]
    return wave, s, amdq, df - amdq


def _pressure(g1, q):
    return g1 * (q[..., 3] - 0.5 * (q[..., 1] * q[..., 1] + q[..., 2] * q[..., 2]) / q[..., 0])


def _euler_roe(g1, ixy, ql, qr):
    mu, mv = ixy, 3 - ixy
    rl, rr = np.sqrt(ql[..., 0]), np.sqrt(qr[..., 0])
    pl, pr = _pressure(g1, ql), _pressure(g1, qr)
    rs = rl + rr
    u = (ql[..., mu] / rl + qr[..., mu] / rr) / rs
    v = (ql[..., mv] / rl + qr[..., mv] / rr) / rs
    enth = ((ql[..., 3] + pl) / rl + (qr[..., 3] + pr) / rr) / rs
    u2v2 = u * u + v * v
    c2 = g1 * (enth - 0.5 * u2v2)
    a = np.sqrt(c2)
    return u, v, enth, u2v2, c2, a, g1 / c2, enth - u2v2, pl, pr


def _rpn2_euler(pd, ixy, ql, qr):
    gamma = pd[0]
    g1 = gamma - 1.0
    efix = pd[1] != 0.0
    mu, mv = ixy, 3 - ixy
    u, v, enth, u2v2, c2, a, g1a2, euv, pl, pr = _euler_roe(g1, ixy, ql, qr)
    d = qr - ql
    a3 = g1a2 * (euv * d[..., 0] + u * d[..., mu] + v * d[..., mv] - d[..., 3])
    a2 = d[..., mv] - v * d[..., 0]
    a4 = (d[..., mu] + (a - u) * d[..., 0] - a * a3) / (2.0 * a)
    a1 = d[..., 0] - a3 - a4
    sh = ql.shape[:-1]
    wave = np.zeros(sh + (4, 4))
    s = np.empty(sh + (4,))
    wave[..., 0, 0] = a1
    wave[..., 0, mu] = a1 * (u - a)
    wave[..., 0, mv] = a1 * v
    wave[..., 0, 3] = a1 * (enth - u * a)
    wave[..., 1, 0] = a3
    wave[..., 1, mu] = a3 * u
    wave[..., 1, mv] = a3 * v
    wave[..., 1, 3] = a3 * 0.5 * u2v2
    wave[..., 2, mv] = a2
    wave[..., 2, 3] = a2 * v
    wave[..., 3, 0] = a4
    wave[..., 3, mu] = a4 * (u + a)
    wave[..., 3, mv] = a4 * v
    wave[..., 3, 3] = a4 * (enth + u * a)
    s[..., 0] = u - a
    s[..., 1] = u
    s[..., 2] = u
    s[..., 3] = u + a
    if not efix:
        amdq = np.zeros(sh + (4,))
        apdq = np.zeros(sh + (4,))
        for p in range(4):
            neg = (s[..., p] < 0.0)[..., None]
            sw = s[..., p, None] * wave[..., p, :]
            amdq = np.where(neg, amdq + sw, amdq)
            apdq = np.where(neg, apdq, apdq + sw)
        return wave, s, amdq, apdq
    s0 = ql[..., mu] / ql[..., 0] - np.sqrt(gamma * pl / ql[..., 0])
    q1 = ql + wave[..., 0, :]
    p1 = g1 * (q1[..., 3] - 0.5 * (q1[..., mu] * q1[..., mu] + q1[..., mv] * q1[..., mv]) / q1[..., 0])
    s1 = q1[..., mu] / q1[..., 0] - np.sqrt(gamma * p1 / q1[..., 0])
    trans1 = (s0 < 0.0) & (s1 > 0.0)
    sf1 = np.where(trans1, s0 * (s1 - s[..., 0]) / (s1 - s0),
                   np.where(s[..., 0] < 0.0, s[..., 0], 0.0))
    amdq = sf1[..., None] * wave[..., 0, :]
    go2 = s[..., 1] < 0.0
    amdq = np.where(go2[..., None], amdq + s[..., 1, None] * wave[..., 1, :], amdq)
    amdq = np.where(go2[..., None], amdq + s[..., 2, None] * wave[..., 2, :], amdq)
    s3 = qr[..., mu] / qr[..., 0] + np.sqrt(gamma * pr / qr[..., 0])
    q2 = qr - wave[..., 3, :]
    p2 = g1 * (q2[..., 3] - 0.5 * (q2[..., mu] * q2[..., mu] + q2[..., mv] * q2[..., mv]) / q2[..., 0])
    s2 = q2[..., mu] / q2[..., 0] + np.sqrt(gamma * p2 / q2[..., 0])
    trans4 = (s2 < 0.0) & (s3 > 0.0)
    sf4 = np.where(trans4, s2 * (s3 - s[..., 3]) / (s3 - s2), s[..., 3])
    add4 = go2 & (trans4 | (s[..., 3] < 0.0))
    amdq = np.where(add4[..., None], amdq + sf4[..., None] * wave[..., 3, :], amdq)
    allright = (s0 >= 0.0) & (s[..., 0] > 0.0)
    amdq = np.where(allright[..., None], 0.0, amdq)
    df = np.zeros_like(amdq)
    for p in range(4):
        df = df + s[..., p, None] * wave[..., p, :]
    return wave, s, amdq, df - amdq


def _split(sb, wb):
    bm = np.zeros(wb.shape[:-2] + (wb.shape[-1],))
    bp = np.zeros_like(bm)
    for p in range(wb.shape[-2]):
        bm = bm + np.minimum(sb[..., p], 0.0)[..., None] * wb[..., p, :]
        bp = bp + np.maximum(sb[..., p], 0.0)[..., None] * wb[..., p, :]
    return bm, bp


def _rpt2_acoustics(pd, ixy, ql, qr, asdq):
    cc, zz = pd[2], pd[3]
    mu, mv = ixy, 3 - ixy
    a1 = (-asdq[..., 0] + zz * asdq[..., mv]) / (2.0 * zz)
    a2 = (asdq[..., 0] + zz * asdq[..., mv]) / (2.0 * zz)
    bm = np.zeros_like(asdq)
    bp = np.zeros_like(asdq)
    bm[..., 0] = cc * a1 * zz
    bm[..., mv] = -cc * a1
    bp[..., 0] = cc * a2 * zz
    bp[..., mv] = cc * a2
    return bm, bp


def _rpt2_shallow(pd, ixy, ql, qr, asdq):
    g = pd[0]
    mu, mv = ixy, 3 - ixy
    hl, hr = ql[..., 0], qr[..., 0]
    hsl, hsr = np.sqrt(hl), np.sqrt(hr)
    hsq2 = hsl + hsr
    u = (ql[..., mu] / hsl + qr[..., mu] / hsr) / hsq2
    v = (ql[..., mv] / hsl + qr[..., mv] / hsr) / hsq2
    c = np.sqrt(g * ((hl + hr) * 0.5))
    a1 = ((v + c) * asdq[..., 0] - asdq[..., mv]) * (0.5 / c)
    a2 = asdq[..., mu] - u * asdq[..., 0]
    a3 = (-(v - c) * asdq[..., 0] + asdq[..., mv]) * (0.5 / c)
    sh = asdq.shape[:-1]
    wb = np.zeros(sh + (3, 3))
    sb = np.empty(sh + (3,))
    wb[..., 0, 0] = a1
    wb[..., 0, mu] = a1 * u
    wb[..., 0, mv] = a1 * (v - c)
    wb[..., 1, mu] = a2
    wb[..., 2, 0] = a3
    wb[..., 2, mu] = a3 * u
    wb[..., 2, mv] = a3 * (v + c)
    sb[..., 0] = v - c
    sb[..., 1] = v
    sb[..., 2] = v + c
    return _split(sb, wb)


def _rpt2_euler(pd, ixy, ql, qr, asdq):
    g1 = pd[0] - 1.0
    mu, mv = ixy, 3 - ixy
    u, v, enth, u2v2, c2, a, g1a2, euv, _, _ = _euler_roe(g1, ixy, ql, qr)
    a3 = g1a2 * (euv * asdq[..., 0] + u * asdq[..., mu] + v * asdq[..., mv] - asdq[..., 3])
    a2 = asdq[..., mu] - u * asdq[..., 0]
    a4 = (asdq[..., mv] + (a - v) * asdq[..., 0] - a * a3) / (2.0 * a)
    a1 = asdq[..., 0] - a3 - a4
    sh = asdq.shape[:-1]
    wb = np.zeros(sh + (4, 4))
    sb = np.empty(sh + (4,))
    wb[..., 0, 0] = a1
    wb[..., 0, mu] = a1 * u
    wb[..., 0, mv] = a1 * (v - a)
    wb[..., 0, 3] = a1 * (enth - v * a)
    wb[..., 1, 0] = a3
    wb[..., 1, mu] = a3 * u
    wb[..., 1, mv] = a3 * v
    wb[..., 1, 3] = a3 * 0.5 * u2v2
    wb[..., 2, mu] = a2
    wb[..., 2, 3] = a2 * u
    wb[..., 3, 0] = a4
    wb[..., 3, mu] = a4 * u
    wb[..., 3, mv] = a4 * (v + a)
    wb[..., 3, 3] = a4 * (enth + v * a)
    sb[..., 0] = v - a
    sb[..., 1] = v
    sb[..., 2] = v
    sb[..., 3] = v + a
    return _split(sb, wb)


RPN2 = {RP_ACOUSTICS: _rpn2_acoustics, RP_SHALLOW: _rpn2_shallow, RP_EULER: _rpn2_euler}
RPT2 = {RP_ACOUSTICS: _rpt2_acoustics, RP_SHALLOW: _rpt2_shallow, RP_EULER: _rpt2_euler}


def philim(lim, r):
    if lim == 1:
        return np.maximum(0.0, np.minimum(1.0, r))
    if lim == 2:
        return np.maximum(0.0, np.maximum(np.minimum(1.0, 2.0 * r), np.minimum(2.0, r)))
    if lim == 3:
        return (r + np.abs(r)) / (1.0 + np.abs(r))
    if lim == 4:
        c = (1.0 + r) / 2.0
        return np.maximum(0.0, np.minimum(c, np.minimum(2.0, 2.0 * r)))
    return np.ones_like(r)


def _sweep(rp, pd, ixy, slices, dtdn, order, tw, mthlim):
    """All slices of one sweep at once.  slices: (ns, n+4, m), cells -2..n+1.
    Returns qadd (ns, n, m), fadd at edges 0..n (ns, n+1, m),
    g1, g2 (ns, n, m) and the max Courant number."""
    ns, n4, m = slices.shape
    n = n4 - 4
    ql = slices[:, 0:n + 3]      # cells -2..n   (left of edges -1..n+1)
    qr = slices[:, 1:n + 4]      # cells -1..n+1 (right of edges -1..n+1)
    with np.errstate(all="ignore"):
        wave, s, amdq, apdq = RPN2[rp](pd, ixy, ql, qr)  # edges -1..n+1 (n+3)
        # edge e at index e+1
        E = slice(1, n + 2)       # edges 0..n
        cfl = float(np.max(np.maximum(dtdn * s[:, E], -dtdn * s[:, E]))) if n >= 0 else 0.0
        qadd = (0.0 - dtdn * apdq[:, 1:n + 1]) - dtdn * amdq[:, 2:n + 2]
        fadd = np.zeros((ns, n + 1, m))
        cq = np.zeros((ns, n + 1, m))
        if order == 2:
            wave = wave.copy()
            mw = wave.shape[-2]
            for p in range(mw):
                lim = mthlim[p]
                if lim == 0:
                    continue
                w = wave[:, :, p, :]  # (ns, n+3, m)
                wn2 = np.zeros(w.shape[:2])
                for k in range(m):
                    wn2 = wn2 + w[..., k] * w[..., k]
                dot = np.zeros((ns, n + 2))  # dot[e+1] = W[e].W[e+1], e=-1..n
                for k in range(m):
                    dot = dot + w[:, 0:n + 2, k] * w[:, 1:n + 3, k]
                dl = dot[:, 0:n + 1]
                dr = dot[:, 1:n + 2]
                wn = wn2[:, E]
                r = np.where(s[:, E, p] > 0.0, dl / wn, dr / wn)
                phi = philim(lim, r)
                lw = np.where((wn == 0.0)[..., None], w[:, E], phi[..., None] * w[:, E])
                wave[:, E, p, :] = lw
            sa = np.abs(s[:, E])
            dtave = 0.5 * (dtdn + dtdn)
            for p in range(mw):
                cq = cq + (sa[..., p] * (1.0 - sa[..., p] * dtave))[..., None] * wave[:, E, p, :]
            fadd = fadd + 0.5 * cq
        g1 = np.zeros((ns, n + 2, m))  # cells -1..n (index c+1)
        g2 = np.zeros((ns, n + 2, m))
        if tw > 0:
            am = amdq[:, E]
            ap = apdq[:, E]
            if order == 2 and tw == 2:
                am = am + cq
                ap = ap - cq
            qlE, qrE = ql[:, E], qr[:, E]
            h = 0.5 * dtdn
            bm, bp = RPT2[rp](pd, ixy, qlE, qrE, am)
            g1[:, 0:n + 1] = g1[:, 0:n + 1] - h * bm   # cell e-1 at index e
            g2[:, 0:n + 1] = g2[:, 0:n + 1] - h * bp
            bm, bp = RPT2[rp](pd, ixy, qlE, qrE, ap)
            g1[:, 1:n + 2] = g1[:, 1:n + 2] - h * bm   # cell e at index e+1
            g2[:, 1:n + 2] = g2[:, 1:n + 2] - h * bp
    return qadd, fadd, g1[:, 1:n + 1], g2[:, 1:n + 1], cfl


def step2(rp, pd, qbc, dx, dy, dt, order=2, tw=2, mthlim=(4, 4, 4, 4)):
    """The unsplit step on qbc (m, mx+4, my+4).  Returns (q_interior, cfl)."""
    m, nx, ny = qbc.shape
    mx, my = nx - 4, ny - 4
    dtdx, dtdy = dt / dx, dt / dy
    pd = list(pd) + [0.0] * (8 - len(pd))
    q = qbc[:, 2:2 + mx, 2:2 + my].copy()
    # x-sweep: slices are rows j = -1..my  -> (ns=my+2, mx+4, m)
    sl = np.ascontiguousarray(np.transpose(qbc[:, :, 1:my + 3], (2, 1, 0)))
    qa, fa, g1, g2, cx = _sweep(rp, pd, 1, sl, dtdx, order, tw, mthlim)
    # to (m, mx, my) layout; slice index t+1 is row t
    T = lambda a: np.transpose(a, (2, 1, 0))
    q = q + dtdy * T(g2[0:my])
    q = q + T(qa[1:my + 1]) - dtdx * (T(fa[1:my + 1, 1:]) - T(fa[1:my + 1, :-1])) \
        - dtdy * (T(g2[1:my + 1]) - T(g1[1:my + 1]))
    q = q - dtdy * T(g1[2:my + 2])
    # y-sweep: slices are columns i = -1..mx -> (ns=mx+2, my+4, m)
    sl = np.ascontiguousarray(np.transpose(qbc[:, 1:mx + 3, :], (1, 2, 0)))
    qa, fa, g1, g2, cy = _sweep(rp, pd, 2, sl, dtdy, order, tw, mthlim)
    U = lambda a: np.transpose(a, (2, 0, 1))
    q = q + dtdx * U(g2[0:mx])
    q = q + U(qa[1:mx + 1]) - dtdy * (U(fa[1:mx + 1, 1:]) - U(fa[1:mx + 1, :-1])) \
        - dtdx * (U(g2[1:mx + 1]) - U(g1[1:mx + 1]))
    q = q - dtdx * U(g1[2:mx + 2])
    return q, max(cx, cy)
