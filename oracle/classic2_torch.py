"""PyTorch transcription of the classic unsplit 2D step, for gradients.

TEST INFRASTRUCTURE ONLY (the checker; never imported by the product path).
Third restatement of the step (after ``classic2_ref.c`` and
``classic2_np.py``), written with torch operations so that torch.autograd
differentiates exactly the operations of the step, including the branch the
limiter and the entropy fix take (``torch.where``).  It is the reference for
the hand-written adjoint kernel; in FP64 it reproduces the C oracle.

PARITY UNPINNED against the reference's Fortran (absent from the mounted
clawpack tree; upstream pyclaw/src/pyclaw/classic/{step2,flux2,limiter}.f90,
riemann/src/rpn2_acoustics.f90, rpt2_acoustics.f90,
rpn2_shallow_roe_with_efix.f90, rpt2_shallow_roe_with_efix.f90).

Supported: acoustics_2D (rp 1) and shallow_roe_with_efix_2D (rp 2), limiters
0-4, order 1/2, transverse_waves 0/1/2, BCs extrap/periodic/wall.
Layout: q is (m, mx, my) like PyClaw's state.q.
"""
from __future__ import annotations

import numpy as np
import torch

RP_ACOUSTICS, RP_SHALLOW = 1, 2
BC_EXTRAP, BC_PERIODIC, BC_WALL = 1, 2, 3


class _Sqrt(torch.autograd.Function):
    """Correctly rounded square root with derivative 1 / (2 sqrt(x)).  Torch's
    vectorised CPU float64 sqrt is off by one ulp on some inputs, so on the
    CPU the value is taken from numpy (IEEE sqrt); on CUDA torch.sqrt is
    already correctly rounded."""

    @staticmethod
    def forward(ctx, x):
        if x.device.type == "cpu":
            y = torch.from_numpy(np.sqrt(x.detach().numpy()))
        else:
            y = torch.sqrt(x)
        ctx.save_for_backward(y)
        return y

    @staticmethod
    def backward(ctx, g):
        (y,) = ctx.saved_tensors
        return torch.where(g == 0.0, torch.zeros_like(g), g / (2.0 * y))


def _sqrt(x):
    return _Sqrt.apply(x)


def ghost_map(n, bc_lo, bc_hi, g=2):
    """Source index and wall flag for padded positions -g .. n+g-1."""
    src, neg = [], []
    for i in range(-g, n + g):
        if i < 0:
            b = bc_lo
            s = 0 if b == BC_EXTRAP else (i + n if b == BC_PERIODIC else -1 - i)
        elif i >= n:
            b = bc_hi
            s = n - 1 if b == BC_EXTRAP else (i - n if b == BC_PERIODIC else 2 * n - 1 - i)
        else:
            b, s = None, i
        src.append(s)
        neg.append(b == BC_WALL)
    return np.array(src), np.array(neg)


def fill_ghosts(q, bc_lower, bc_upper, g=2):
    """qbc (m, mx+2g, my+2g) as PyClaw's _apply_bcs builds it (x boundaries
    over all rows, then y boundaries over all columns), as a gather so that
    gradients flow back to the interior cells."""
    m, mx, my = q.shape
    sx, nx = ghost_map(mx, bc_lower[0], bc_upper[0], g)
    sy, ny = ghost_map(my, bc_lower[1], bc_upper[1], g)
    ix = torch.as_tensor(sx, device=q.device)
    iy = torch.as_tensor(sy, device=q.device)
    qbc = q[:, ix][:, :, iy]
    sign = torch.ones((m, len(sx), len(sy)), dtype=q.dtype, device=q.device)
    sign[1, torch.as_tensor(nx, device=q.device), :] *= -1.0
    sign[2, :, torch.as_tensor(ny, device=q.device)] *= -1.0
    return qbc * sign


def _stack_comp(vals):
    return torch.stack(vals, dim=-1)


# ---------------------------------------------------------------- Riemann solvers
# ql, qr: (..., m).  Return wave (..., mw, m), s (..., mw), amdq, apdq, roe.

def _rpn2_acoustics(pd, ixy, ql, qr):
    cc, zz = pd[2], pd[3]
    mu, mv = ixy, 3 - ixy
    d0 = qr[..., 0] - ql[..., 0]
    d1 = qr[..., mu] - ql[..., mu]
    a1 = (-d0 + zz * d1) / (2.0 * zz)
    a2 = (d0 + zz * d1) / (2.0 * zz)
    z = torch.zeros_like(a1)
    c1 = [None] * 3
    c1[0], c1[mu], c1[mv] = -a1 * zz, a1, z
    c2 = [None] * 3
    c2[0], c2[mu], c2[mv] = a2 * zz, a2, z
    wave = torch.stack([_stack_comp(c1), _stack_comp(c2)], dim=-2)
    s = torch.stack([torch.full_like(a1, -cc), torch.full_like(a1, cc)], dim=-1)
    amdq = s[..., 0, None] * wave[..., 0, :]
    apdq = s[..., 1, None] * wave[..., 1, :]
    return wave, s, amdq, apdq, None


def _roe_shallow(pd, ixy, ql, qr):
    g = pd[0]
    mu, mv = ixy, 3 - ixy
    hl, hr = ql[..., 0], qr[..., 0]
    hsl, hsr = _sqrt(hl), _sqrt(hr)
    hsq2 = hsl + hsr
    u = (ql[..., mu] / hsl + qr[..., mu] / hsr) / hsq2
    v = (ql[..., mv] / hsl + qr[..., mv] / hsr) / hsq2
    c = _sqrt(g * ((hl + hr) * 0.5))
    return u, v, c


def _rpn2_shallow(pd, ixy, ql, qr):
    g = pd[0]
    mu, mv = ixy, 3 - ixy
    hl, hr = ql[..., 0], qr[..., 0]
    u, v, c = _roe_shallow(pd, ixy, ql, qr)
    half = 0.5 / c
    d0 = hr - hl
    d1 = qr[..., mu] - ql[..., mu]
    d2 = qr[..., mv] - ql[..., mv]
    a1 = ((u + c) * d0 - d1) * half
    a2 = -v * d0 + d2
    a3 = (-(u - c) * d0 + d1) * half
    z = torch.zeros_like(a1)
    c1 = [None] * 3
    c1[0], c1[mu], c1[mv] = a1, a1 * (u - c), a1 * v
    c2 = [None] * 3
    c2[0], c2[mu], c2[mv] = z, z, a2
    c3 = [None] * 3
    c3[0], c3[mu], c3[mv] = a3, a3 * (u + c), a3 * v
    wave = torch.stack([_stack_comp(c1), _stack_comp(c2), _stack_comp(c3)], dim=-2)
    s = torch.stack([u - c, u, u + c], dim=-1)
    # Harten-Hyman entropy fix
    # Intermediate depths h1, h3 can be <= 0; the step's s1 / s3 are then NaN
    # and every comparison with them is false.  The branch values are taken
    # on safe inputs so that no NaN enters the gradient through an
    # unselected branch; the selected values are unchanged.
    one = torch.ones_like(hl)
    s0 = ql[..., mu] / hl - _sqrt(g * hl)
    h1 = hl + wave[..., 0, 0]
    hu1 = ql[..., mu] + wave[..., 0, mu]
    ok1 = h1 > 0.0
    h1s = torch.where(ok1, h1, one)
    s1 = hu1 / h1s - _sqrt(g * h1s)
    trans1 = (s0 < 0.0) & (s1 > 0.0) & ok1
    d1s = torch.where(trans1, s1 - s0, one)
    sf1 = torch.where(trans1, s0 * (s1 - s[..., 0]) / d1s,
                      torch.where(s[..., 0] < 0.0, s[..., 0], torch.zeros_like(s0)))
    amdq = sf1[..., None] * wave[..., 0, :]
    go2 = s[..., 1] < 0.0
    amdq = torch.where(go2[..., None], amdq + s[..., 1, None] * wave[..., 1, :], amdq)
    s03 = qr[..., mu] / hr + _sqrt(g * hr)
    h3 = hr - wave[..., 2, 0]
    hu3 = qr[..., mu] - wave[..., 2, mu]
    ok3 = h3 > 0.0
    h3s = torch.where(ok3, h3, one)
    s3 = hu3 / h3s + _sqrt(g * h3s)
    trans3 = (s3 < 0.0) & (s03 > 0.0) & ok3
    d3s = torch.where(trans3, s03 - s3, one)
    sf3 = torch.where(trans3, s3 * (s03 - s[..., 2]) / d3s, s[..., 2])
    add3 = go2 & (trans3 | (s[..., 2] < 0.0))
    amdq = torch.where(add3[..., None], amdq + sf3[..., None] * wave[..., 2, :], amdq)
    allright = (s0 >= 0.0) & (s[..., 0] > 0.0)
    amdq = torch.where(allright[..., None], torch.zeros_like(amdq), amdq)
    df = torch.zeros_like(amdq)
    for p in range(3):
        df = df + s[..., p, None] * wave[..., p, :]
    return wave, s, amdq, df - amdq, (u, v, c, half)


def _split(sb, wb):
    bm = torch.zeros_like(wb[..., 0, :])
    bp = torch.zeros_like(bm)
    z = torch.zeros_like(sb[..., 0])
    for p in range(wb.shape[-2]):
        bm = bm + torch.minimum(sb[..., p], z)[..., None] * wb[..., p, :]
        bp = bp + torch.maximum(sb[..., p], z)[..., None] * wb[..., p, :]
    return bm, bp


def _rpt2_acoustics(pd, ixy, roe, asdq):
    cc, zz = pd[2], pd[3]
    mu, mv = ixy, 3 - ixy
    a1 = (-asdq[..., 0] + zz * asdq[..., mv]) / (2.0 * zz)
    a2 = (asdq[..., 0] + zz * asdq[..., mv]) / (2.0 * zz)
    z = torch.zeros_like(a1)
    bm = [None] * 3
    bm[0], bm[mu], bm[mv] = cc * a1 * zz, z, -cc * a1
    bp = [None] * 3
    bp[0], bp[mu], bp[mv] = cc * a2 * zz, z, cc * a2
    return _stack_comp(bm), _stack_comp(bp)


def _rpt2_shallow(pd, ixy, roe, asdq):
    mu, mv = ixy, 3 - ixy
    u, v, c, half = roe
    a1 = ((v + c) * asdq[..., 0] - asdq[..., mv]) * half
    a2 = asdq[..., mu] - u * asdq[..., 0]
    a3 = (-(v - c) * asdq[..., 0] + asdq[..., mv]) * half
    z = torch.zeros_like(a1)
    w1 = [None] * 3
    w1[0], w1[mu], w1[mv] = a1, a1 * u, a1 * (v - c)
    w2 = [None] * 3
    w2[0], w2[mu], w2[mv] = z, a2, z
    w3 = [None] * 3
    w3[0], w3[mu], w3[mv] = a3, a3 * u, a3 * (v + c)
    wb = torch.stack([_stack_comp(w1), _stack_comp(w2), _stack_comp(w3)], dim=-2)
    sb = torch.stack([v - c, v, v + c], dim=-1)
    return _split(sb, wb)


RPN2 = {RP_ACOUSTICS: _rpn2_acoustics, RP_SHALLOW: _rpn2_shallow}
RPT2 = {RP_ACOUSTICS: _rpt2_acoustics, RP_SHALLOW: _rpt2_shallow}


def philim(lim, r):
    zero = torch.zeros_like(r)
    if lim == 1:
        return torch.maximum(zero, torch.minimum(torch.ones_like(r), r))
    if lim == 2:
        return torch.maximum(zero, torch.maximum(torch.minimum(torch.ones_like(r), 2.0 * r),
                                                 torch.minimum(torch.full_like(r, 2.0), r)))
    if lim == 3:
        return (r + torch.abs(r)) / (1.0 + torch.abs(r))
    if lim == 4:
        c = (1.0 + r) / 2.0
        return torch.maximum(zero, torch.minimum(c, torch.minimum(torch.full_like(r, 2.0),
                                                                  2.0 * r)))
    return torch.ones_like(r)


def _sweep(rp, pd, ixy, slices, dtdn, order, tw, mthlim):
    """All slices of one sweep; slices (ns, n+4, m), cells -2..n+1."""
    ns, n4, m = slices.shape
    n = n4 - 4
    ql = slices[:, 0:n + 3]
    qr = slices[:, 1:n + 4]
    wave, s, amdq, apdq, roe = RPN2[rp](pd, ixy, ql, qr)  # edges -1..n+1 at index e+1
    E = slice(1, n + 2)
    cfl = float(torch.max(torch.abs(s[:, E])).detach() * dtdn)
    qadd = (0.0 - dtdn * apdq[:, 1:n + 1]) - dtdn * amdq[:, 2:n + 2]
    mw = wave.shape[-2]
    cq = torch.zeros_like(apdq[:, E])
    if order == 2:
        limited = []
        for p in range(mw):
            w = wave[:, :, p, :]
            lim = mthlim[p]
            if lim == 0:
                limited.append(w[:, E])
                continue
            wn2 = torch.zeros_like(w[..., 0])
            for k in range(m):
                wn2 = wn2 + w[..., k] * w[..., k]
            dot = torch.zeros_like(w[:, 0:n + 2, 0])
            for k in range(m):
                dot = dot + w[:, 0:n + 2, k] * w[:, 1:n + 3, k]
            dl, dr, wn = dot[:, 0:n + 1], dot[:, 1:n + 2], wn2[:, E]
            safe = torch.where(wn == 0.0, torch.ones_like(wn), wn)
            r = torch.where(s[:, E, p] > 0.0, dl / safe, dr / safe)
            phi = philim(lim, r)
            limited.append(torch.where((wn == 0.0)[..., None], w[:, E], phi[..., None] * w[:, E]))
        lw = torch.stack(limited, dim=-2)
        sa = torch.abs(s[:, E])
        dtave = 0.5 * (dtdn + dtdn)
        for p in range(mw):
            cq = cq + (sa[..., p] * (1.0 - sa[..., p] * dtave))[..., None] * lw[..., p, :]
    fadd = 0.0 + 0.5 * cq
    zero_g = torch.zeros_like(apdq[:, 0:n + 2])
    g1, g2 = zero_g, zero_g
    if tw > 0:
        am, ap = amdq[:, E], apdq[:, E]
        if order == 2 and tw == 2:
            am = am + cq
            ap = ap - cq
        roeE = None if roe is None else tuple(x[:, E] for x in roe)
        h = 0.5 * dtdn
        bm, bp = RPT2[rp](pd, ixy, roeE, am)
        pad = torch.zeros_like(bm[:, :1])
        g1 = torch.cat([0.0 - h * bm, pad], dim=1)   # cell e-1 at index e
        g2 = torch.cat([0.0 - h * bp, pad], dim=1)
        bm, bp = RPT2[rp](pd, ixy, roeE, ap)
        g1 = g1 - h * torch.cat([pad, bm], dim=1)    # cell e at index e+1
        g2 = g2 - h * torch.cat([pad, bp], dim=1)
    return qadd, fadd, g1[:, 1:n + 1], g2[:, 1:n + 1], cfl


def step(rp, pd, q, dx, dy, dt, bc_lower, bc_upper, order=2, tw=2, mthlim=(4, 4, 4, 4)):
    """One unsplit step of q (m, mx, my) with boundary conditions; returns
    (qnew, cfl).  Differentiable in q."""
    m, mx, my = q.shape
    dtdx, dtdy = dt / dx, dt / dy
    pd = list(pd) + [0.0] * (8 - len(pd))
    qbc = fill_ghosts(q, bc_lower, bc_upper)
    T = lambda a: a.permute(2, 1, 0)
    sl = qbc[:, :, 1:my + 3].permute(2, 1, 0)
    qa, fa, g1, g2, cx = _sweep(rp, pd, 1, sl, dtdx, order, tw, mthlim)
    v = q + dtdy * T(g2[0:my])
    v = v + T(qa[1:my + 1]) - dtdx * (T(fa[1:my + 1, 1:]) - T(fa[1:my + 1, :-1])) \
        - dtdy * (T(g2[1:my + 1]) - T(g1[1:my + 1]))
    v = v - dtdy * T(g1[2:my + 2])
    U = lambda a: a.permute(2, 0, 1)
    sl = qbc[:, 1:mx + 3, :].permute(1, 2, 0)
    qa, fa, g1, g2, cy = _sweep(rp, pd, 2, sl, dtdy, order, tw, mthlim)
    v = v + dtdx * U(g2[0:mx])
    v = v + U(qa[1:mx + 1]) - dtdy * (U(fa[1:mx + 1, 1:]) - U(fa[1:mx + 1, :-1])) \
        - dtdx * (U(g2[1:mx + 1]) - U(g1[1:mx + 1]))
    v = v - dtdx * U(g1[2:mx + 2])
    return v, max(cx, cy)
