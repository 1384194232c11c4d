/*
 * classic3_ref.c -- CPU oracle for the classic unsplit 3D wave-propagation
 * step (PyClaw ClawSolver3D, classic3).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py may load it.
 * The product path (clawpack_gb300) never links or calls it.
 *
 * PARITY UNPINNED.  The reference code of this path lives in the empty
 * pyclaw and riemann submodules of the mounted clawpack 5.14.0 tree
 * (.gitmodules:1-21; meson.build:62-76); the upstream files it corresponds
 * to are pyclaw/src/pyclaw/classic/step3.f90, flux3.f90 and
 * riemann/src/rpn3_acoustics.f90, rpt3_acoustics.f90, rptt3_acoustics.f90 and
 * rpn3_euler.f90, rpt3_euler.f90, rptt3_euler.f90.
 * This is a restatement, in original code, of the published method the
 * reference cites for it (CITATION.md:46-58): J. O. Langseth and R. J.
 * LeVeque, "A wave propagation method for three-dimensional hyperbolic
 * conservation laws", J. Comput. Phys. 165 (2000) 126-166.
 *
 * The method.  Each direction d in turn (x, y, z) sweeps 1D slices along d;
 * t1 = (d+1) mod 3 and t2 = (d+2) mod 3 are the transverse directions.  At
 * every edge of a slice:
 *   - rpn3 gives waves W_p, speeds s_p and the fluctuations A-dQ, A+dQ;
 *     A-+dQ update the two edge cells (first-order Godunov terms);
 *   - with order 2 the waves are limited as in 2D and the correction flux
 *     F = 1/2 sum_p |s_p| (1 - |s_p| dt/dn) W~_p is added;
 *   - transverse_waves = 10 * a + b: a >= 1 splits each fluctuation (A-dQ
 *     into the cell before the edge, A+dQ into the cell after it; with a = 2
 *     after the correction flux is folded into them) in t1 by rpt3 into
 *     B-+ and in t2 into C-+, which enter the transverse fluxes G (faces
 *     normal to t1) and H (faces normal to t2) of that cell with -1/2 dt/dn;
 *     b >= 1 splits B-+ again in t2 and C-+ in t1 by rptt3 (corner
 *     transport): a part C+B moving up in t2 moves 1/6 dt^2/(dn dt2) of the
 *     G flux from the face's own t2 row to the row above, C-B to the row
 *     below, and likewise for H.  For constant-coefficient advection with
 *     order 1 and transverse_waves 11 this is exactly the corner transport
 *     upwind scheme (trilinear upwind interpolation); the 1/6 makes the six
 *     orderings of the three directions add up to the third-order
 *     cross-derivative term dt^3 u v w q_xyz of the Taylor expansion.
 * Supported transverse_waves: 0, 10, 11, 20, 22.
 *
 * Floating-point order.  Each slice's outputs are formed edge by edge in the
 * order the serial flux3 loops would (the chain of a fluctuation as one
 * value per flux entry: the single transverse term, then the corner terms);
 * the per-cell accumulation then adds, sweep by sweep, the contributions of
 * the 3x3 slices around the cell with t2 outer and t1 inner.  Built with
 * -ffp-contract=off.
 *
 * Layout: q with ghost cells is (m, mx+4, my+4, mz+4), Fortran order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RP3_ACOUSTICS 1
#define RP3_EULER 2
#define RP3_ADVECTION 100 /* constant-velocity advection: a known-answer solver */

#define BC_EXTRAP 1
#define BC_PERIODIC 2
#define BC_WALL 3

#define MAXM 5
#define MAXW 5
#define ERR_ARG -1
#define ERR_ALLOC -3

typedef struct {
    int id, m, mw;
    double pd[8];
} rp3_t;

static int rp3_shape(int id, int *m, int *mw)
{
    switch (id) {
    case RP3_ACOUSTICS: *m = 4; *mw = 2; return 0;
    case RP3_EULER: *m = 5; *mw = 3; return 0;
    case RP3_ADVECTION: *m = 1; *mw = 1; return 0;
    default: return ERR_ARG;
    }
}

/* ------------------------------------------------------------------------
 * Riemann solvers.  d, t: axes 0, 1, 2.  Acoustics q = (p, u, v, w) with
 * pd = (rho, bulk, c, Z = rho c); the velocity along axis a is q[1 + a].
 * Advection q = (q) with pd = (u, v, w).
 * ---------------------------------------------------------------------- */
/* 3D Euler, q = (rho, rho u, rho v, rho w, E), pd = (gamma): the Roe state
 * of an edge (square-root-density averages of the velocity and the total
 * enthalpy; FVMHP sec. 15.3) and the decomposition of a vector along axis d
 * into three waves: acoustic (u_d - a), the entropy and the two shear waves
 * together (u_d), acoustic (u_d + a) (upstream rpn3_euler.f90, which uses
 * the same three families; no entropy fix). */
typedef struct {
    double u[3], enth, a, g1a2, euv, u2;
    int bad;
} roe3_t;

static double euler3_pressure(double gamma1, const double *q)
{
    return gamma1 * (q[4] - 0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / q[0]);
}

static void roe3(const rp3_t *rp, const double *ql, const double *qr, roe3_t *R)
{
    const double gamma1 = rp->pd[0] - 1.0;
    double rhsqrtl = sqrt(ql[0]), rhsqrtr = sqrt(qr[0]);
    double pl = euler3_pressure(gamma1, ql);
    double pr = euler3_pressure(gamma1, qr);
    double rhsq2 = rhsqrtl + rhsqrtr;
    for (int k = 0; k < 3; k++) R->u[k] = (ql[1 + k] / rhsqrtl + qr[1 + k] / rhsqrtr) / rhsq2;
    R->enth = ((ql[4] + pl) / rhsqrtl + (qr[4] + pr) / rhsqrtr) / rhsq2;
    R->u2 = R->u[0] * R->u[0] + R->u[1] * R->u[1] + R->u[2] * R->u[2];
    double c2 = gamma1 * (R->enth - 0.5 * R->u2);
    R->bad = !(c2 > 0.0);
    R->a = sqrt(c2);
    R->g1a2 = gamma1 / c2;
    R->euv = R->enth - R->u2;
}

static void roe3_waves(const roe3_t *R, int d, const double *dq, double *w, double *s)
{
    const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
    const int mn = 1 + d, m1 = 1 + t1, m2 = 1 + t2;
    const double un = R->u[d], v1 = R->u[t1], v2 = R->u[t2], a = R->a, enth = R->enth;
    double a2 = R->g1a2 * (R->euv * dq[0] + un * dq[mn] + v1 * dq[m1] + v2 * dq[m2] - dq[4]);
    double a3 = dq[m1] - v1 * dq[0];
    double a4 = dq[m2] - v2 * dq[0];
    double a5 = (dq[mn] + (a - un) * dq[0] - a * a2) / (2.0 * a);
    double a1 = dq[0] - a2 - a5;
    double *w1 = w, *w2 = w + 5, *w3 = w + 10;
    w1[0] = a1; w1[mn] = a1 * (un - a); w1[m1] = a1 * v1; w1[m2] = a1 * v2;
    w1[4] = a1 * (enth - un * a);
    s[0] = un - a;
    w2[0] = a2; w2[mn] = a2 * un; w2[m1] = a2 * v1 + a3; w2[m2] = a2 * v2 + a4;
    w2[4] = a2 * 0.5 * R->u2 + a3 * v1 + a4 * v2;
    s[1] = un;
    w3[0] = a5; w3[mn] = a5 * (un + a); w3[m1] = a5 * v1; w3[m2] = a5 * v2;
    w3[4] = a5 * (enth + un * a);
    s[2] = un + a;
}

static int rpn3(const rp3_t *rp, int d, const double *ql, const double *qr, double *wave,
                double *s, double *amdq, double *apdq)
{
    if (rp->id == RP3_EULER) {
        roe3_t R;
        roe3(rp, ql, qr, &R);
        double dq[5];
        for (int k = 0; k < 5; k++) dq[k] = qr[k] - ql[k];
        roe3_waves(&R, d, dq, wave, s);
        for (int k = 0; k < 5; k++) amdq[k] = apdq[k] = 0.0;
        for (int p = 0; p < 3; p++)
            for (int k = 0; k < 5; k++) {
                if (s[p] < 0.0)
                    amdq[k] = amdq[k] + s[p] * wave[5 * p + k];
                else
                    apdq[k] = apdq[k] + s[p] * wave[5 * p + k];
            }
        return R.bad;
    }
    if (rp->id == RP3_ADVECTION) {
        const double u = rp->pd[d];
        wave[0] = qr[0] - ql[0];
        s[0] = u;
        amdq[0] = fmin(u, 0.0) * wave[0];
        apdq[0] = fmax(u, 0.0) * wave[0];
        return 0;
    }
    const double cc = rp->pd[2], zz = rp->pd[3];
    const int mn = 1 + d;
    double d0 = qr[0] - ql[0];
    double d1 = qr[mn] - ql[mn];
    double a1 = (-d0 + zz * d1) / (2.0 * zz);
    double a2 = (d0 + zz * d1) / (2.0 * zz);
    double *w1 = wave, *w2 = wave + 4;
    for (int k = 0; k < 4; k++) w1[k] = w2[k] = 0.0;
    w1[0] = -a1 * zz; w1[mn] = a1;
    s[0] = -cc;
    w2[0] = a2 * zz; w2[mn] = a2;
    s[1] = cc;
    for (int k = 0; k < 4; k++) {
        amdq[k] = s[0] * w1[k];
        apdq[k] = s[1] * w2[k];
    }
    return 0;
}

/* Split asdq along axis t into the parts moving down (bm) and up (bp);
 * ql / qr: the states of the normal edge (Euler: its Roe state). */
static void rpt3(const rp3_t *rp, int t, const double *ql, const double *qr,
                 const double *asdq, double *bm, double *bp)
{
    if (rp->id == RP3_EULER) {
        roe3_t R;
        roe3(rp, ql, qr, &R);
        double w[15], sb[3];
        roe3_waves(&R, t, asdq, w, sb);
        for (int k = 0; k < 5; k++) {
            double lo = 0.0, hi = 0.0;
            for (int p = 0; p < 3; p++) {
                lo = lo + fmin(sb[p], 0.0) * w[5 * p + k];
                hi = hi + fmax(sb[p], 0.0) * w[5 * p + k];
            }
            bm[k] = lo;
            bp[k] = hi;
        }
        return;
    }
    if (rp->id == RP3_ADVECTION) {
        const double v = rp->pd[t];
        bm[0] = fmin(v, 0.0) * asdq[0];
        bp[0] = fmax(v, 0.0) * asdq[0];
        return;
    }
    const double cc = rp->pd[2], zz = rp->pd[3];
    const int mt = 1 + t;
    double a1 = (-asdq[0] + zz * asdq[mt]) / (2.0 * zz);
    double a2 = (asdq[0] + zz * asdq[mt]) / (2.0 * zz);
    for (int k = 0; k < 4; k++) bm[k] = bp[k] = 0.0;
    bm[0] = cc * a1 * zz; bm[mt] = -cc * a1;
    bp[0] = cc * a2 * zz; bp[mt] = cc * a2;
}

/* Split a transverse fluctuation (already split along axis t1) along axis
 * t2, with the eigenstructure of the normal edge's state along t2: rpt3
 * along t2 (upstream rptt3_*.f90 use the same Roe state). */
static void rptt3(const rp3_t *rp, int t1, int t2, const double *ql, const double *qr,
                  const double *bsasdq, double *cm, double *cp)
{
    (void)t1;
    rpt3(rp, t2, ql, qr, bsasdq, cm, cp);
}

static double philim3(int id, double r)
{
    double c;
    switch (id) {
    case 1: return fmax(0.0, fmin(1.0, r));
    case 2: return fmax(0.0, fmax(fmin(1.0, 2.0 * r), fmin(2.0, r)));
    case 3: return (r + fabs(r)) / (1.0 + fabs(r));
    case 4:
        c = (1.0 + r) / 2.0;
        return fmax(0.0, fmin(c, fmin(2.0, 2.0 * r)));
    default: return 1.0;
    }
}

/* Outputs of one slice, per cell position c (offset 2 in the arrays):
 *   qadd[c]            first-order update (times dt/dn)
 *   fadd[c]            correction flux at edge c (between cells c-1, c)
 *   G[c][s][o]         flux through the t1-face s (0: a-1/2, 1: a+1/2) of
 *                      cell c at t2-offset o-1 from the slice
 *   H[c][s][o]         flux through the t2-face s (0: b-1/2, 1: b+1/2) at
 *                      t1-offset o-1
 * Each array holds M values per entry. */
typedef struct {
    double *qadd, *fadd, *G, *H;
} slice_out;

#define NGH 6 /* 2 faces x 3 offsets */

typedef struct {
    double *q1d, *wave, *s, *amdq, *apdq, *cq;
} work3_t;

/* The chain of one fluctuation asdq: single transverse split and, with
 * double transverse, the corner terms; g[s][o] and h[s][o] are the values
 * it adds to the flux entries of the receiving cell. */
static void chain(const rp3_t *rp, int t1, int t2, const double *ql, const double *qr,
                  const double *asdq, int dbl, double h, double f1, double f2, double *g,
                  double *hh)
{
    const int m = rp->m;
    double bm[MAXM], bp[MAXM], cm[MAXM], cp[MAXM];
    rpt3(rp, t1, ql, qr, asdq, bm, bp);
    rpt3(rp, t2, ql, qr, asdq, cm, cp);
    for (int e = 0; e < NGH * m; e++) g[e] = hh[e] = 0.0;
#define GE(s, o, k) g[((s) * 3 + (o)) * m + (k)]
#define HE(s, o, k) hh[((s) * 3 + (o)) * m + (k)]
    for (int k = 0; k < m; k++) {
        GE(0, 1, k) = 0.0 - h * bm[k];
        GE(1, 1, k) = 0.0 - h * bp[k];
        HE(0, 1, k) = 0.0 - h * cm[k];
        HE(1, 1, k) = 0.0 - h * cp[k];
    }
    if (!dbl) return;
    double cmb[MAXM], cpb[MAXM];
    for (int s = 0; s < 2; s++) {
        rptt3(rp, t1, t2, ql, qr, s ? bp : bm, cmb, cpb);
        for (int k = 0; k < m; k++) {
            GE(s, 1, k) = GE(s, 1, k) + f2 * (cpb[k] - cmb[k]);
            GE(s, 2, k) = 0.0 - f2 * cpb[k];
            GE(s, 0, k) = 0.0 + f2 * cmb[k];
        }
    }
    for (int s = 0; s < 2; s++) {
        rptt3(rp, t2, t1, ql, qr, s ? cp : cm, cmb, cpb);
        for (int k = 0; k < m; k++) {
            HE(s, 1, k) = HE(s, 1, k) + f1 * (cpb[k] - cmb[k]);
            HE(s, 2, k) = 0.0 - f1 * cpb[k];
            HE(s, 0, k) = 0.0 + f1 * cmb[k];
        }
    }
#undef GE
#undef HE
}

/* One slice of n cells along direction d (cells -2..n+1 in q1d). */
static double flux3_slice(const rp3_t *rp, int d, int n, double dtdn, double dtt1, double dtt2,
                          int order, int tw, const int *mthlim, const work3_t *wk,
                          const slice_out *out, int *bad)
{
    const int m = rp->m, mw = rp->mw, off = 2;
    const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
    const int single = tw / 10, dbl = tw % 10;
    int e, k, p;
#define Q(c) (wk->q1d + (size_t)((c) + off) * m)
#define W(e) (wk->wave + (size_t)((e) + off) * mw * m)
#define S(e) (wk->s + (size_t)((e) + off) * mw)
#define AM(e) (wk->amdq + (size_t)((e) + off) * m)
#define AP(e) (wk->apdq + (size_t)((e) + off) * m)
#define CQ(e) (wk->cq + (size_t)((e) + off) * m)
#define QA(c) (out->qadd + (size_t)((c) + off) * m)
#define FA(c) (out->fadd + (size_t)((c) + off) * m)
#define GG(c) (out->G + (size_t)((c) + off) * NGH * m)
#define HH(c) (out->H + (size_t)((c) + off) * NGH * m)
    for (e = -1; e <= n + 1; e++) *bad |= rpn3(rp, d, Q(e - 1), Q(e), W(e), S(e), AM(e), AP(e));
    for (e = -2; e <= n + 1; e++) {
        for (k = 0; k < m; k++) QA(e)[k] = FA(e)[k] = CQ(e)[k] = 0.0;
        for (k = 0; k < NGH * m; k++) GG(e)[k] = HH(e)[k] = 0.0;
    }
    for (e = 0; e <= n; e++)
        for (k = 0; k < m; k++) {
            QA(e)[k] = QA(e)[k] - dtdn * AP(e)[k];
            QA(e - 1)[k] = QA(e - 1)[k] - dtdn * AM(e)[k];
        }
    double cfl = 0.0;
    for (e = 0; e <= n; e++)
        for (p = 0; p < mw; p++) cfl = fmax(cfl, fmax(dtdn * S(e)[p], -dtdn * S(e)[p]));

    if (order == 2) {
        for (p = 0; p < mw; p++) {
            if (mthlim[p] == 0) continue;
            double dotr = 0.0;
            for (e = -1; e <= n; e++) {
                double wnorm2 = 0.0, dotl = dotr;
                dotr = 0.0;
                const double *we = W(e) + p * m, *wn = W(e + 1) + p * m;
                for (k = 0; k < m; k++) {
                    wnorm2 = wnorm2 + we[k] * we[k];
                    dotr = dotr + we[k] * wn[k];
                }
                if (e == -1) continue;
                if (wnorm2 == 0.0) continue;
                double r = (S(e)[p] > 0.0) ? dotl / wnorm2 : dotr / wnorm2;
                double phi = philim3(mthlim[p], r);
                for (k = 0; k < m; k++) W(e)[p * m + k] = phi * W(e)[p * m + k];
            }
        }
        const double dtave = 0.5 * (dtdn + dtdn);
        for (e = 0; e <= n; e++)
            for (k = 0; k < m; k++) {
                double c = 0.0;
                for (p = 0; p < mw; p++) {
                    double sa = fabs(S(e)[p]);
                    c = c + sa * (1.0 - sa * dtave) * W(e)[p * m + k];
                }
                CQ(e)[k] = c;
                FA(e)[k] = FA(e)[k] + 0.5 * c;
            }
    }

    if (single > 0) {
        if (order == 2 && single == 2)
            for (e = 0; e <= n; e++)
                for (k = 0; k < m; k++) {
                    AM(e)[k] = AM(e)[k] + CQ(e)[k];
                    AP(e)[k] = AP(e)[k] - CQ(e)[k];
                }
        const double h = 0.5 * dtdn;
        const double sixth = 1.0 / 6.0;
        const double f1 = sixth * dtdn * dtt1, f2 = sixth * dtdn * dtt2;
        double g[NGH * MAXM], hh[NGH * MAXM];
        /* A-dQ enters the cell before the edge, A+dQ the cell after it */
        for (e = 0; e <= n; e++) {
            chain(rp, t1, t2, Q(e - 1), Q(e), AM(e), dbl, h, f1, f2, g, hh);
            for (k = 0; k < NGH * m; k++) {
                GG(e - 1)[k] = GG(e - 1)[k] + g[k];
                HH(e - 1)[k] = HH(e - 1)[k] + hh[k];
            }
        }
        for (e = 0; e <= n; e++) {
            chain(rp, t1, t2, Q(e - 1), Q(e), AP(e), dbl, h, f1, f2, g, hh);
            for (k = 0; k < NGH * m; k++) {
                GG(e)[k] = GG(e)[k] + g[k];
                HH(e)[k] = HH(e)[k] + hh[k];
            }
        }
    }
#undef Q
#undef W
#undef S
#undef AM
#undef AP
#undef CQ
#undef QA
#undef FA
#undef GG
#undef HH
    return cfl;
}

/* ------------------------------------------------------------------------
 * Ghost fill (PyClaw's _apply_bcs in 3D): x over every (y, z) row including
 * ghosts, then y, then z.  Walls mirror and negate the normal velocity,
 * component 1 + axis (acoustics); for m = 1 nothing is negated.
 * ---------------------------------------------------------------------- */
int gclaw3_ref_fill_ghosts(int m, int mx, int my, int mz, int g, const int *bc_lower,
                           const int *bc_upper, const double *q, double *qbc)
{
    if (m < 1 || m > MAXM || g < 1 || mx < g || my < g || mz < g) return ERR_ARG;
    const int n[3] = {mx, my, mz};
    const int nb[3] = {mx + 2 * g, my + 2 * g, mz + 2 * g};
    for (int d = 0; d < 3; d++)
        if (bc_lower[d] < BC_EXTRAP || bc_lower[d] > BC_WALL || bc_upper[d] < BC_EXTRAP ||
            bc_upper[d] > BC_WALL)
            return ERR_ARG;
#define QB(k, i, j, l) \
    qbc[(size_t)(k) + (size_t)m * ((size_t)(i) + (size_t)nb[0] * ((size_t)(j) + (size_t)nb[1] * (size_t)(l)))]
    for (int l = 0; l < mz; l++)
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++)
                for (int k = 0; k < m; k++)
                    QB(k, i + g, j + g, l + g) =
                        q[(size_t)k + (size_t)m * ((size_t)i + (size_t)mx * ((size_t)j + (size_t)my * l))];
    for (int d = 0; d < 3; d++) {
        const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
        for (int b = 0; b < nb[t2]; b++)
            for (int a = 0; a < nb[t1]; a++)
                for (int gl = 0; gl < g; gl++) {
                    int src[2], neg[2] = {0, 0};
                    switch (bc_lower[d]) {
                    case BC_EXTRAP: src[0] = g; break;
                    case BC_PERIODIC: src[0] = gl + n[d]; break;
                    default: src[0] = 2 * g - 1 - gl; neg[0] = 1; break;
                    }
                    switch (bc_upper[d]) {
                    case BC_EXTRAP: src[1] = g + n[d] - 1; break;
                    case BC_PERIODIC: src[1] = g + gl; break;
                    default: src[1] = g + n[d] - 1 - gl; neg[1] = 1; break;
                    }
                    const int dst[2] = {gl, g + n[d] + gl};
                    for (int side = 0; side < 2; side++) {
                        int is[3], id[3];
                        is[d] = src[side]; is[t1] = a; is[t2] = b;
                        id[d] = dst[side]; id[t1] = a; id[t2] = b;
                        for (int k = 0; k < m; k++) {
                            double v = QB(k, is[0], is[1], is[2]);
                            if (neg[side] && m > 1 && k == 1 + d) v = -v;
                            QB(k, id[0], id[1], id[2]) = v;
                        }
                    }
                }
    }
#undef QB
    return 0;
}

/* The unsplit 3D step on ghost-filled arrays (m, mx+4, my+4, mz+4); qnew
 * receives qold plus all updates. */
static int step3_dirs(int rp_id, const double *pd, int mx, int my, int mz, const double *qold,
                      double *qnew, double dx, double dy, double dz, double dt, int order,
                      int tw, const int *mthlim, double *cfl_out, int nthreads, int d_lo,
                      int d_hi);

int gclaw3_ref_step3(int rp_id, const double *pd, int mx, int my, int mz, const double *qold,
                     double *qnew, double dx, double dy, double dz, double dt, int order, int tw,
                     const int *mthlim, double *cfl_out, int nthreads)
{
    return step3_dirs(rp_id, pd, mx, my, mz, qold, qnew, dx, dy, dz, dt, order, tw, mthlim,
                      cfl_out, nthreads, 0, 2);
}

/* The sweep of one direction d (0, 1, 2) alone, without transverse terms:
 * one stage of PyClaw's dimensionally split 3D step (classic3 step3ds,
 * upstream pyclaw/src/pyclaw/classic/step3ds.f90), on ghost-filled arrays. */
int gclaw3_ref_step3ds(int rp_id, const double *pd, int mx, int my, int mz, const double *qold,
                       double *qnew, double dx, double dy, double dz, double dt, int order,
                       const int *mthlim, int d, double *cfl_out, int nthreads)
{
    if (d < 0 || d > 2) return ERR_ARG;
    return step3_dirs(rp_id, pd, mx, my, mz, qold, qnew, dx, dy, dz, dt, order, 0, mthlim,
                      cfl_out, nthreads, d, d);
}

static int step3_dirs(int rp_id, const double *pd, int mx, int my, int mz, const double *qold,
                      double *qnew, double dx, double dy, double dz, double dt, int order,
                      int tw, const int *mthlim, double *cfl_out, int nthreads, int d_lo,
                      int d_hi)
{
    rp3_t rp;
    rp.id = rp_id;
    if (rp3_shape(rp_id, &rp.m, &rp.mw) || mx < 2 || my < 2 || mz < 2) return ERR_ARG;
    if (order < 1 || order > 2) return ERR_ARG;
    if (tw != 0 && tw != 10 && tw != 11 && tw != 20 && tw != 22) return ERR_ARG;
    memcpy(rp.pd, pd, sizeof rp.pd);
    const int m = rp.m, mw = rp.mw, g = 2;
    const int n[3] = {mx, my, mz};
    const int nb[3] = {mx + 4, my + 4, mz + 4};
    const double dtd[3] = {dt / dx, dt / dy, dt / dz};
    memcpy(qnew, qold, sizeof(double) * (size_t)m * nb[0] * nb[1] * nb[2]);
    if (nthreads < 1) nthreads = 1;
    const int nmax = (mx > my ? (mx > mz ? mx : mz) : (my > mz ? my : mz)) + 4;
    const size_t per = (size_t)nmax * m;
    double cfl = 0.0;
    int rc = 0, bad = 0;
#define QI(arr, k, i, j, l) \
    (arr)[(size_t)(k) + (size_t)m * ((size_t)(i) + (size_t)nb[0] * ((size_t)(j) + (size_t)nb[1] * (size_t)(l)))]

    for (int d = d_lo; d <= d_hi && rc == 0; d++) {
        const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
        const int nd = n[d], n1 = n[t1], n2 = n[t2];
        const int ns1 = n1 + 2, ns2 = n2 + 2; /* slices a = -1..n1, b = -1..n2 */
        const size_t nsl = (size_t)ns1 * ns2;
        double *QA = malloc(sizeof(double) * per * nsl);
        double *FA = malloc(sizeof(double) * per * nsl);
        double *GA = malloc(sizeof(double) * per * NGH * nsl);
        double *HA = malloc(sizeof(double) * per * NGH * nsl);
        double *cfls = malloc(sizeof(double) * nsl);
        if (!QA || !FA || !GA || !HA || !cfls) {
            free(QA); free(FA); free(GA); free(HA); free(cfls);
            rc = ERR_ALLOC;
            break;
        }
#pragma omp parallel num_threads(nthreads) reduction(| : bad)
        {
            work3_t wk;
            wk.q1d = malloc(sizeof(double) * per);
            wk.wave = malloc(sizeof(double) * (size_t)nmax * mw * m);
            wk.s = malloc(sizeof(double) * (size_t)nmax * mw);
            wk.amdq = malloc(sizeof(double) * per);
            wk.apdq = malloc(sizeof(double) * per);
            wk.cq = malloc(sizeof(double) * per);
#pragma omp for schedule(static)
            for (long sl = 0; sl < (long)nsl; sl++) {
                const int a = (int)(sl % ns1) - 1, b = (int)(sl / ns1) - 1;
                for (int c = -2; c < nd + 2; c++) {
                    int ii[3];
                    ii[d] = c + g; ii[t1] = a + g; ii[t2] = b + g;
                    for (int k = 0; k < m; k++)
                        wk.q1d[(size_t)(c + 2) * m + k] = QI(qold, k, ii[0], ii[1], ii[2]);
                }
                slice_out so = {QA + per * sl, FA + per * sl, GA + per * NGH * sl,
                                HA + per * NGH * sl};
                cfls[sl] = flux3_slice(&rp, d, nd, dtd[d], dtd[t1], dtd[t2], order, tw, mthlim,
                                       &wk, &so, &bad);
            }
            free(wk.q1d); free(wk.wave); free(wk.s); free(wk.amdq); free(wk.apdq); free(wk.cq);
        }
        for (size_t sl = 0; sl < nsl; sl++) cfl = fmax(cfl, cfls[sl]);

        /* ordered accumulation: slices b = B-1..B+1 (outer), a = A-1..A+1 */
        const double dtn = dtd[d], dt1 = dtd[t1], dt2 = dtd[t2];
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (long cell = 0; cell < (long)n1 * n2; cell++) {
            const int A = (int)(cell % n1), B = (int)(cell / n1);
            for (int c = 0; c < nd; c++) {
                int ii[3];
                ii[d] = c + g; ii[t1] = A + g; ii[t2] = B + g;
                for (int db = -1; db <= 1; db++)
                    for (int da = -1; da <= 1; da++) {
                        const int a = A - da, b = B - db;
                        const size_t sl = (size_t)(a + 1) + (size_t)ns1 * (size_t)(b + 1);
                        const double *qa = QA + per * sl + (size_t)(c + 2) * m;
                        const double *fa0 = FA + per * sl + (size_t)(c + 2) * m;
                        const double *fa1 = fa0 + m;
                        const double *G = GA + per * NGH * sl + (size_t)(c + 2) * NGH * m;
                        const double *H = HA + per * NGH * sl + (size_t)(c + 2) * NGH * m;
                        for (int k = 0; k < m; k++) {
                            double v = QI(qnew, k, ii[0], ii[1], ii[2]);
#define GV(s, o) G[((s) * 3 + (o) + 1) * m + k]
#define HV(s, o) H[((s) * 3 + (o) + 1) * m + k]
                            if (da == 0 && db == 0) {
                                v = v + qa[k] - dtn * (fa1[k] - fa0[k]) -
                                    dt1 * (GV(1, 0) - GV(0, 0)) - dt2 * (HV(1, 0) - HV(0, 0));
                            } else {
                                const double gt = da == 0 ? 0.0 - dt1 * (GV(1, db) - GV(0, db))
                                                  : da == 1 ? dt1 * GV(1, db)
                                                            : 0.0 - dt1 * GV(0, db);
                                const double ht = db == 0 ? 0.0 - dt2 * (HV(1, da) - HV(0, da))
                                                  : db == 1 ? dt2 * HV(1, da)
                                                            : 0.0 - dt2 * HV(0, da);
                                v = v + gt + ht;
                            }
#undef GV
#undef HV
                            QI(qnew, k, ii[0], ii[1], ii[2]) = v;
                        }
                    }
            }
        }
        free(QA); free(FA); free(GA); free(HA); free(cfls);
    }
#undef QI
    *cfl_out = cfl;
    if (rc == 0 && bad) rc = 2; /* non-physical state (Euler: c^2 <= 0) */
    return rc;
}

/* Ghost fill + step on interior-shaped arrays (m, mx, my, mz). */
int gclaw3_ref_step(int rp_id, const double *pd, int mx, int my, int mz, const double *q,
                    double *qout, double dx, double dy, double dz, double dt, int order, int tw,
                    const int *mthlim, const int *bc_lower, const int *bc_upper,
                    double *cfl_out, int nthreads)
{
    int m, mw;
    if (rp3_shape(rp_id, &m, &mw)) return ERR_ARG;
    const int nx = mx + 4, ny = my + 4, nz = mz + 4;
    const size_t nb = (size_t)m * nx * ny * nz;
    double *qa = malloc(sizeof(double) * nb), *qb = malloc(sizeof(double) * nb);
    if (!qa || !qb) {
        free(qa); free(qb);
        return ERR_ALLOC;
    }
    int rc = gclaw3_ref_fill_ghosts(m, mx, my, mz, 2, bc_lower, bc_upper, q, qa);
    if (rc == 0)
        rc = gclaw3_ref_step3(rp_id, pd, mx, my, mz, qa, qb, dx, dy, dz, dt, order, tw, mthlim,
                              cfl_out, nthreads);
    if (rc == 0 || rc == 2)
        for (int l = 0; l < mz; l++)
            for (int j = 0; j < my; j++)
                for (int i = 0; i < mx; i++)
                    for (int k = 0; k < m; k++)
                        qout[(size_t)k + (size_t)m * ((size_t)i + (size_t)mx * ((size_t)j + (size_t)my * l))] =
                            qb[(size_t)k + (size_t)m * ((size_t)(i + 2) + (size_t)nx * ((size_t)(j + 2) + (size_t)ny * (l + 2)))];
    free(qa);
    free(qb);
    return rc;
}

int gclaw3_ref_shape(int rp_id, int *m, int *mw) { return rp3_shape(rp_id, m, mw); }

/* One 3D Riemann problem along axis d (0, 1, 2), for known-answer tests. */
int gclaw3_ref_rpn3(int rp_id, const double *pd, int d, const double *ql, const double *qr,
                    double *wave, double *s, double *amdq, double *apdq)
{
    rp3_t rp;
    rp.id = rp_id;
    if (rp3_shape(rp_id, &rp.m, &rp.mw) || d < 0 || d > 2) return ERR_ARG;
    memcpy(rp.pd, pd, sizeof rp.pd);
    return rpn3(&rp, d, ql, qr, wave, s, amdq, apdq) ? 2 : 0;
}

/* PyClaw's dimensionally split 3D step (Godunov splitting, ClawSolver3D's
 * default dimensional_split = True): boundary conditions and the x-sweep,
 * boundary conditions again on its result and the y-sweep, then the
 * z-sweep; *cfl_out is the largest of the three sweeps' Courant numbers.
 * Interior-shaped arrays (m, mx, my, mz). */
int gclaw3_ref_step_split(int rp_id, const double *pd, int mx, int my, int mz, const double *q,
                          double *qout, double dx, double dy, double dz, double dt, int order,
                          const int *mthlim, const int *bc_lower, const int *bc_upper,
                          double *cfl_out, int nthreads)
{
    int m, mw;
    if (rp3_shape(rp_id, &m, &mw)) return ERR_ARG;
    const int nx = mx + 4, ny = my + 4, nz = mz + 4;
    const size_t nb = (size_t)m * nx * ny * nz, ni = (size_t)m * mx * my * mz;
    double *qa = malloc(sizeof(double) * nb), *qb = malloc(sizeof(double) * nb);
    double *qi = malloc(sizeof(double) * ni);
    if (!qa || !qb || !qi) {
        free(qa); free(qb); free(qi);
        return ERR_ALLOC;
    }
    memcpy(qi, q, sizeof(double) * ni);
    double cfl = 0.0;
    int rc = 0, bad = 0;
    for (int d = 0; d < 3; d++) {
        double c = 0.0;
        rc = gclaw3_ref_fill_ghosts(m, mx, my, mz, 2, bc_lower, bc_upper, qi, qa);
        if (rc) break;
        rc = gclaw3_ref_step3ds(rp_id, pd, mx, my, mz, qa, qb, dx, dy, dz, dt, order, mthlim, d,
                                &c, nthreads);
        if (rc == 2) bad = 1;
        else if (rc) break;
        rc = 0;
        cfl = cfl > c ? cfl : c;
        for (int l = 0; l < mz; l++)
            for (int j = 0; j < my; j++)
                for (int i = 0; i < mx; i++)
                    for (int k = 0; k < m; k++)
                        qi[(size_t)k + (size_t)m * ((size_t)i + (size_t)mx * ((size_t)j + (size_t)my * l))] =
                            qb[(size_t)k + (size_t)m * ((size_t)(i + 2) + (size_t)nx * ((size_t)(j + 2) + (size_t)ny * (l + 2)))];
    }
    if (rc == 0) memcpy(qout, qi, sizeof(double) * ni);
    free(qa); free(qb); free(qi);
    *cfl_out = cfl;
    if (rc) return rc;
    return bad ? 2 : 0;
}
