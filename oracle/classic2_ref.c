/*
 * classic2_ref.c -- CPU oracle for the PyClaw classic unsplit 2D step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py may load it.
 * The product path (clawpack_gb300) never links or calls it.
 *
 * PARITY UNPINNED.  The reference (clawpack 5.14.0, umbrella repository)
 * declares the code of this path in git submodules that are empty in the
 * mounted tree (.gitmodules:1-21; meson.build:62-76 maps 'pyclaw' to
 * pyclaw/src and 'riemann' to riemann).  The files this oracle follows are the
 * upstream ones, absent here:
 *     pyclaw/src/pyclaw/classic/step2.f90     (step2: the unsplit 2D step)
 *     pyclaw/src/pyclaw/classic/flux2.f90     (flux2: one 1D slice)
 *     pyclaw/src/pyclaw/classic/limiter.f90   (wave limiter + philim)
 *     pyclaw/src/pyclaw/solver.py             (_apply_bcs ghost fill)
 *     riemann/src/rpn2_acoustics.f90,  rpt2_acoustics.f90
 *     riemann/src/rpn2_shallow_roe_with_efix.f90, rpt2_shallow_roe_with_efix.f90
 *     riemann/src/rpn2_euler_4wave.f90, rpt2_euler.f90
 *     riemann/src/rpn2_vc_acoustics.f90, rpt2_vc_acoustics.f90
 *     riemann/src/rpn2_shallow_bathymetry_fwave.f90 (f-wave solver)
 * It is a restatement, in original code, of the published method that the
 * reference names as its algorithm source (CITATION.md:19-41):
 * R. J. LeVeque, J. Comput. Phys. 131 (1997) 327-353, and LeVeque, "Finite
 * Volume Methods for Hyperbolic Problems" (2002), ch. 6 (limiters), ch. 15
 * (Roe solvers, Harten-Hyman entropy fix), ch. 19-21 (unsplit 2D method with
 * transverse propagation of fluctuations and of correction waves).
 *
 * Floating-point order.  Every accumulation is written in the order the
 * serial Fortran step performs it (slice by slice, x-sweep then y-sweep,
 * each qnew(i,j) receiving the row j-1, j, j+1 terms of the x-sweep and then
 * the column i-1, i, i+1 terms of the y-sweep).  Build with
 * -ffp-contract=off so that no multiply-add is fused.  The slices are
 * independent, so they run in parallel (OpenMP) with per-slice outputs and a
 * separate ordered accumulation pass; the arithmetic per cell is unchanged.
 *
 * Memory layout: q with ghost cells is PyClaw's qbc, shape
 * (num_eqn, mx+2g, my+2g) in Fortran order, i.e. the component index varies
 * fastest, then x, then y.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RP_ACOUSTICS 1
#define RP_SHALLOW_ROE_EFIX 2
#define RP_EULER_4WAVE 3
#define RP_VC_ACOUSTICS 4
#define RP_SHALLOW_BATHY_FWAVE 5

#define BC_CUSTOM 0
#define BC_EXTRAP 1
#define BC_PERIODIC 2
#define BC_WALL 3

#define MAXM 4
#define MAXW 4

#define ERR_ARG -1
#define ERR_ALLOC -3
#define ERR_NONPHYSICAL 2

typedef struct {
    int id, m, mw;
    double pd[8];
} rp_t;

static int rp_shape(int id, int *m, int *mw)
{
    switch (id) {
    case RP_ACOUSTICS: *m = 3; *mw = 2; return 0;
    case RP_SHALLOW_ROE_EFIX: *m = 3; *mw = 3; return 0;
    case RP_EULER_4WAVE: *m = 4; *mw = 4; return 0;
    case RP_VC_ACOUSTICS: *m = 3; *mw = 2; return 0;
    case RP_SHALLOW_BATHY_FWAVE: *m = 3; *mw = 3; return 0;
    default: return ERR_ARG;
    }
}

/* ------------------------------------------------------------------------
 * Normal Riemann solvers.  ql = state of the cell left of the edge (cell e-1),
 * qr = state of the cell right of it (cell e).  ixy = 1 for an x-edge,
 * 2 for a y-edge; mu is the normal momentum/velocity component, mv the
 * transverse one.  wave is [mw][m], s is [mw].
 * Returns nonzero for a non-physical state (negative Euler sound speed
 * squared), which upstream stops on.
 * ---------------------------------------------------------------------- */

/* Constant-coefficient acoustics, q = (p, u, v); eigenvalues -c, +c with
 * eigenvectors (-Z, 1, 0) and (Z, 1, 0) in (p, normal u, transverse u),
 * Z = rho c (upstream rpn2_acoustics.f90). */
static int rpn2_acoustics(const rp_t *rp, int ixy, const double *ql, const double *qr,
                          double *wave, double *s, double *amdq, double *apdq)
{
    const double cc = rp->pd[2], zz = rp->pd[3];
    const int mu = ixy, mv = 3 - ixy;
    double d0 = qr[0] - ql[0];
    double d1 = qr[mu] - ql[mu];
    double a1 = (-d0 + zz * d1) / (2.0 * zz);
    double a2 = (d0 + zz * d1) / (2.0 * zz);
    double *w1 = wave, *w2 = wave + 3;
    w1[0] = -a1 * zz; w1[mu] = a1; w1[mv] = 0.0;
    s[0] = -cc;
    w2[0] = a2 * zz; w2[mu] = a2; w2[mv] = 0.0;
    s[1] = cc;
    for (int k = 0; k < 3; k++) {
        amdq[k] = s[0] * w1[k];
        apdq[k] = s[1] * w2[k];
    }
    return 0;
}

/* Shallow water Roe solver, q = (h, hu, hv), with the Harten-Hyman entropy
 * fix for transonic rarefactions (FVMHP sec. 15.3.5; upstream
 * rpn2_shallow_roe_with_efix.f90). */
static int rpn2_shallow(const rp_t *rp, int ixy, const double *ql, const double *qr,
                        double *wave, double *s, double *amdq, double *apdq)
{
    const double g = rp->pd[0];
    const int mu = ixy, mv = 3 - ixy;
    double hl = ql[0], hr = qr[0];
    double hsqrtl = sqrt(hl), hsqrtr = sqrt(hr);
    double hsq2 = hsqrtl + hsqrtr;
    double ubar = (ql[mu] / hsqrtl + qr[mu] / hsqrtr) / hsq2;
    double vbar = (ql[mv] / hsqrtl + qr[mv] / hsqrtr) / hsq2;
    double hbar = (hl + hr) * 0.5;
    double cbar = sqrt(g * hbar);
    double d0 = hr - hl, d1 = qr[mu] - ql[mu], d2 = qr[mv] - ql[mv];
    double a1 = ((ubar + cbar) * d0 - d1) * (0.5 / cbar);
    double a2 = -vbar * d0 + d2;
    double a3 = (-(ubar - cbar) * d0 + d1) * (0.5 / cbar);
    double *w1 = wave, *w2 = wave + 3, *w3 = wave + 6;
    w1[0] = a1; w1[mu] = a1 * (ubar - cbar); w1[mv] = a1 * vbar;
    s[0] = ubar - cbar;
    w2[0] = 0.0; w2[mu] = 0.0; w2[mv] = a2;
    s[1] = ubar;
    w3[0] = a3; w3[mu] = a3 * (ubar + cbar); w3[mv] = a3 * vbar;
    s[2] = ubar + cbar;

    /* entropy fix: left-going part amdq, then apdq = (sum s W) - amdq */
    double sfract;
    int k;
    double s0 = ql[mu] / hl - sqrt(g * hl);          /* u - c left of the 1-wave */
    if (s0 >= 0.0 && s[0] > 0.0) {
        for (k = 0; k < 3; k++) amdq[k] = 0.0;       /* fully right-going */
        goto done;
    }
    {
        double h1 = hl + w1[0];
        double hu1 = ql[mu] + w1[mu];
        double s1 = hu1 / h1 - sqrt(g * h1);         /* u - c right of the 1-wave */
        if (s0 < 0.0 && s1 > 0.0)
            sfract = s0 * (s1 - s[0]) / (s1 - s0);   /* transonic 1-rarefaction */
        else if (s[0] < 0.0)
            sfract = s[0];
        else
            sfract = 0.0;
    }
    for (k = 0; k < 3; k++) amdq[k] = sfract * w1[k];
    if (s[1] >= 0.0) goto done;
    for (k = 0; k < 3; k++) amdq[k] = amdq[k] + s[1] * w2[k];
    {
        double s03 = qr[mu] / hr + sqrt(g * hr);     /* u + c right of the 3-wave */
        double h3 = hr - w3[0];
        double hu3 = qr[mu] - w3[mu];
        double s3 = hu3 / h3 + sqrt(g * h3);         /* u + c left of the 3-wave */
        if (s3 < 0.0 && s03 > 0.0)
            sfract = s3 * (s03 - s[2]) / (s03 - s3); /* transonic 3-rarefaction */
        else if (s[2] < 0.0)
            sfract = s[2];
        else
            goto done;
    }
    for (k = 0; k < 3; k++) amdq[k] = amdq[k] + sfract * w3[k];
done:
    for (k = 0; k < 3; k++) {
        double df = 0.0;
        for (int p = 0; p < 3; p++) df = df + s[p] * wave[3 * p + k];
        apdq[k] = df - amdq[k];
    }
    return 0;
}

static double euler_pressure(double gamma1, const double *q)
{
    return gamma1 * (q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0]);
}

/* 2D Euler Roe solver with 4 waves: acoustic (u-c), entropy (u), shear (u),
 * acoustic (u+c); q = (rho, rho u, rho v, E); optional Harten-Hyman entropy
 * fix (pd[1] != 0).  Upstream rpn2_euler_4wave.f90. */
static int rpn2_euler(const rp_t *rp, int ixy, const double *ql, const double *qr,
                      double *wave, double *s, double *amdq, double *apdq)
{
    const double gamma = rp->pd[0], gamma1 = gamma - 1.0;
    const int efix = rp->pd[1] != 0.0;
    const int mu = ixy, mv = 3 - ixy;
    double rhsqrtl = sqrt(ql[0]), rhsqrtr = sqrt(qr[0]);
    double pl = euler_pressure(gamma1, ql);
    double pr = euler_pressure(gamma1, qr);
    double rhsq2 = rhsqrtl + rhsqrtr;
    double u = (ql[mu] / rhsqrtl + qr[mu] / rhsqrtr) / rhsq2;
    double v = (ql[mv] / rhsqrtl + qr[mv] / rhsqrtr) / rhsq2;
    double enth = ((ql[3] + pl) / rhsqrtl + (qr[3] + pr) / rhsqrtr) / rhsq2;
    double u2v2 = u * u + v * v;
    double c2 = gamma1 * (enth - 0.5 * u2v2);
    int bad = !(c2 > 0.0);
    double a = sqrt(c2);
    double g1a2 = gamma1 / c2;
    double euv = enth - u2v2;
    double d0 = qr[0] - ql[0], dmu = qr[mu] - ql[mu], dmv = qr[mv] - ql[mv], d3 = qr[3] - ql[3];
    double a3 = g1a2 * (euv * d0 + u * dmu + v * dmv - d3);
    double a2 = dmv - v * d0;
    double a4 = (dmu + (a - u) * d0 - a * a3) / (2.0 * a);
    double a1 = d0 - a3 - a4;
    double *w1 = wave, *w2 = wave + 4, *w3 = wave + 8, *w4 = wave + 12;
    w1[0] = a1; w1[mu] = a1 * (u - a); w1[mv] = a1 * v; w1[3] = a1 * (enth - u * a);
    s[0] = u - a;
    w2[0] = a3; w2[mu] = a3 * u; w2[mv] = a3 * v; w2[3] = a3 * 0.5 * u2v2;
    s[1] = u;
    w3[0] = 0.0; w3[mu] = 0.0; w3[mv] = a2; w3[3] = a2 * v;
    s[2] = u;
    w4[0] = a4; w4[mu] = a4 * (u + a); w4[mv] = a4 * v; w4[3] = a4 * (enth + u * a);
    s[3] = u + a;

    int k, p;
    if (!efix) {
        for (k = 0; k < 4; k++) {
            amdq[k] = 0.0;
            apdq[k] = 0.0;
        }
        for (p = 0; p < 4; p++) {
            for (k = 0; k < 4; k++) {
                if (s[p] < 0.0)
                    amdq[k] = amdq[k] + s[p] * wave[4 * p + k];
                else
                    apdq[k] = apdq[k] + s[p] * wave[4 * p + k];
            }
        }
        return bad;
    }
    double sfract;
    {
        double cim1 = sqrt(gamma * pl / ql[0]);
        double s0 = ql[mu] / ql[0] - cim1;           /* u - c left of the 1-wave */
        if (s0 >= 0.0 && s[0] > 0.0) {
            for (k = 0; k < 4; k++) amdq[k] = 0.0;
            goto done;
        }
        double rho1 = ql[0] + w1[0];
        double rhou1 = ql[mu] + w1[mu];
        double rhov1 = ql[mv] + w1[mv];
        double en1 = ql[3] + w1[3];
        double p1 = gamma1 * (en1 - 0.5 * (rhou1 * rhou1 + rhov1 * rhov1) / rho1);
        double c1 = sqrt(gamma * p1 / rho1);
        double s1 = rhou1 / rho1 - c1;               /* u - c right of the 1-wave */
        if (s0 < 0.0 && s1 > 0.0)
            sfract = s0 * (s1 - s[0]) / (s1 - s0);
        else if (s[0] < 0.0)
            sfract = s[0];
        else
            sfract = 0.0;
    }
    for (k = 0; k < 4; k++) amdq[k] = sfract * w1[k];
    if (s[1] >= 0.0) goto done;
    for (k = 0; k < 4; k++) amdq[k] = amdq[k] + s[1] * w2[k];
    for (k = 0; k < 4; k++) amdq[k] = amdq[k] + s[2] * w3[k];
    {
        double ci = sqrt(gamma * pr / qr[0]);
        double s3 = qr[mu] / qr[0] + ci;             /* u + c right of the 4-wave */
        double rho2 = qr[0] - w4[0];
        double rhou2 = qr[mu] - w4[mu];
        double rhov2 = qr[mv] - w4[mv];
        double en2 = qr[3] - w4[3];
        double p2 = gamma1 * (en2 - 0.5 * (rhou2 * rhou2 + rhov2 * rhov2) / rho2);
        double cc2 = sqrt(gamma * p2 / rho2);
        double s2 = rhou2 / rho2 + cc2;              /* u + c left of the 4-wave */
        if (s2 < 0.0 && s3 > 0.0)
            sfract = s2 * (s3 - s[3]) / (s3 - s2);
        else if (s[3] < 0.0)
            sfract = s[3];
        else
            goto done;
    }
    for (k = 0; k < 4; k++) amdq[k] = amdq[k] + sfract * w4[k];
done:
    for (k = 0; k < 4; k++) {
        double df = 0.0;
        for (p = 0; p < 4; p++) df = df + s[p] * wave[4 * p + k];
        apdq[k] = df - amdq[k];
    }
    return bad;
}

/* Variable-coefficient acoustics, q = (p, u, v), aux = (rho, c) per cell:
 * the interface Riemann problem between impedances Zl = rho_l c_l and
 * Zr = rho_r c_r (FVMHP sec. 9.9; upstream rpn2_vc_acoustics.f90): speeds
 * -c_l and +c_r, eigenvectors (-Zl, 1, 0) and (Zr, 1, 0).  With equal
 * coefficients on both sides every expression equals rpn2_acoustics'. */
static int rpn2_vc_acoustics(int ixy, const double *ql, const double *qr, const double *al,
                             const double *ar, double *wave, double *s, double *amdq,
                             double *apdq)
{
    const int mu = ixy, mv = 3 - ixy;
    double d0 = qr[0] - ql[0];
    double d1 = qr[mu] - ql[mu];
    double zl = al[0] * al[1], zr = ar[0] * ar[1];
    double a1 = (-d0 + zr * d1) / (zl + zr);
    double a2 = (d0 + zl * d1) / (zl + zr);
    double *w1 = wave, *w2 = wave + 3;
    w1[0] = -a1 * zl; w1[mu] = a1; w1[mv] = 0.0;
    s[0] = -al[1];
    w2[0] = a2 * zr; w2[mu] = a2; w2[mv] = 0.0;
    s[1] = ar[1];
    for (int k = 0; k < 3; k++) {
        amdq[k] = s[0] * w1[k];
        apdq[k] = s[1] * w2[k];
    }
    return 0;
}

/* Shallow water over bathymetry b = aux[0], f-wave form (Bale, LeVeque,
 * Mitran and Rossmanith, SIAM J. Sci. Comput. 24 (2002) 955-978; FVMHP
 * sec. 15.5; upstream rpn2_shallow_bathymetry_fwave.f90): the flux
 * difference plus the bathymetry source, delta = f(qr) - f(ql) +
 * (0, g hbar (br - bl), 0), is split into f-waves Z_p = beta_p r_p along the
 * eigenvectors of the Roe matrix (the Roe averages of rpn2_shallow).
 * amdq / apdq sum the f-waves of negative / positive speed (half each at
 * speed zero).  A still lake (h + b constant, u = v = 0) has delta = 0, so
 * it stays at rest.  Dry or negative depths are non-physical here. */
static int rpn2_shallow_fwave(const rp_t *rp, int ixy, const double *ql, const double *qr,
                              const double *al, const double *ar, double *wave, double *s,
                              double *amdq, double *apdq)
{
    const double g = rp->pd[0];
    const int mu = ixy, mv = 3 - ixy;
    double hl = ql[0], hr = qr[0];
    if (!(hl > 0.0) || !(hr > 0.0)) {
        for (int k = 0; k < 9; k++) wave[k] = 0.0;
        for (int k = 0; k < 3; k++) s[k] = amdq[k] = apdq[k] = 0.0;
        return 1;
    }
    double hsqrtl = sqrt(hl), hsqrtr = sqrt(hr);
    double hsq2 = hsqrtl + hsqrtr;
    double ubar = (ql[mu] / hsqrtl + qr[mu] / hsqrtr) / hsq2;
    double vbar = (ql[mv] / hsqrtl + qr[mv] / hsqrtr) / hsq2;
    double hbar = (hl + hr) * 0.5;
    double cbar = sqrt(g * hbar);
    double ul = ql[mu] / hl, vl = ql[mv] / hl, ur = qr[mu] / hr, vr = qr[mv] / hr;
    double d0 = qr[mu] - ql[mu];
    double d1 = (qr[mu] * ur + 0.5 * g * hr * hr) - (ql[mu] * ul + 0.5 * g * hl * hl) +
                g * hbar * (ar[0] - al[0]);
    double d2 = qr[mu] * vr - ql[mu] * vl;
    s[0] = ubar - cbar;
    s[1] = ubar;
    s[2] = ubar + cbar;
    double b1 = (s[2] * d0 - d1) / (s[2] - s[0]);
    double b3 = (d1 - s[0] * d0) / (s[2] - s[0]);
    double b2 = d2 - vbar * d0;
    double *z1 = wave, *z2 = wave + 3, *z3 = wave + 6;
    z1[0] = b1; z1[mu] = b1 * s[0]; z1[mv] = b1 * vbar;
    z2[0] = 0.0; z2[mu] = 0.0; z2[mv] = b2;
    z3[0] = b3; z3[mu] = b3 * s[2]; z3[mv] = b3 * vbar;
    for (int k = 0; k < 3; k++) amdq[k] = apdq[k] = 0.0;
    for (int p = 0; p < 3; p++)
        for (int k = 0; k < 3; k++) {
            if (s[p] < 0.0) {
                amdq[k] = amdq[k] + wave[3 * p + k];
            } else if (s[p] > 0.0) {
                apdq[k] = apdq[k] + wave[3 * p + k];
            } else {
                amdq[k] = amdq[k] + 0.5 * wave[3 * p + k];
                apdq[k] = apdq[k] + 0.5 * wave[3 * p + k];
            }
        }
    return 0;
}

/* al / ar: aux of the cells left / right of the edge (solvers with aux). */
static int rpn2(const rp_t *rp, int ixy, const double *ql, const double *qr,
                const double *al, const double *ar, double *wave, double *s, double *amdq,
                double *apdq)
{
    switch (rp->id) {
    case RP_ACOUSTICS: return rpn2_acoustics(rp, ixy, ql, qr, wave, s, amdq, apdq);
    case RP_SHALLOW_ROE_EFIX: return rpn2_shallow(rp, ixy, ql, qr, wave, s, amdq, apdq);
    case RP_VC_ACOUSTICS: return rpn2_vc_acoustics(ixy, ql, qr, al, ar, wave, s, amdq, apdq);
    case RP_SHALLOW_BATHY_FWAVE:
        return rpn2_shallow_fwave(rp, ixy, ql, qr, al, ar, wave, s, amdq, apdq);
    default: return rpn2_euler(rp, ixy, ql, qr, wave, s, amdq, apdq);
    }
}

/* ------------------------------------------------------------------------
 * Transverse Riemann solvers: split the normal fluctuation asdq at the edge
 * between ql and qr into the parts going down (bmasdq) and up (bpasdq) in
 * the transverse direction, with the transverse eigenstructure at the
 * edge's Roe state.  bm[k] = sum_p min(sb_p,0) Wb_p[k], bp likewise with max.
 * ---------------------------------------------------------------------- */
static void rpt2_acoustics(const rp_t *rp, int ixy, const double *ql, const double *qr,
                           const double *asdq, double *bm, double *bp)
{
    (void)ql; (void)qr;
    const double cc = rp->pd[2], zz = rp->pd[3];
    const int mu = ixy, mv = 3 - ixy;
    double a1 = (-asdq[0] + zz * asdq[mv]) / (2.0 * zz);
    double a2 = (asdq[0] + zz * asdq[mv]) / (2.0 * zz);
    bm[0] = cc * a1 * zz; bm[mu] = 0.0; bm[mv] = -cc * a1;
    bp[0] = cc * a2 * zz; bp[mu] = 0.0; bp[mv] = cc * a2;
}

static void split_sum(int m, int mw, const double *sb, const double *wb, double *bm, double *bp)
{
    for (int k = 0; k < m; k++) {
        double lo = 0.0, hi = 0.0;
        for (int p = 0; p < mw; p++) {
            lo = lo + fmin(sb[p], 0.0) * wb[m * p + k];
            hi = hi + fmax(sb[p], 0.0) * wb[m * p + k];
        }
        bm[k] = lo;
        bp[k] = hi;
    }
}

static void rpt2_shallow(const rp_t *rp, int ixy, const double *ql, const double *qr,
                         const double *asdq, double *bm, double *bp)
{
    const double g = rp->pd[0];
    const int mu = ixy, mv = 3 - ixy;
    double hl = ql[0], hr = qr[0];
    double hsqrtl = sqrt(hl), hsqrtr = sqrt(hr);
    double hsq2 = hsqrtl + hsqrtr;
    double ubar = (ql[mu] / hsqrtl + qr[mu] / hsqrtr) / hsq2;
    double vbar = (ql[mv] / hsqrtl + qr[mv] / hsqrtr) / hsq2;
    double hbar = (hl + hr) * 0.5;
    double cbar = sqrt(g * hbar);
    double a1 = ((vbar + cbar) * asdq[0] - asdq[mv]) * (0.5 / cbar);
    double a2 = asdq[mu] - ubar * asdq[0];
    double a3 = (-(vbar - cbar) * asdq[0] + asdq[mv]) * (0.5 / cbar);
    double wb[9], sb[3];
    wb[0] = a1; wb[mu] = a1 * ubar; wb[mv] = a1 * (vbar - cbar);
    sb[0] = vbar - cbar;
    wb[3] = 0.0; wb[3 + mu] = a2; wb[3 + mv] = 0.0;
    sb[1] = vbar;
    wb[6] = a3; wb[6 + mu] = a3 * ubar; wb[6 + mv] = a3 * (vbar + cbar);
    sb[2] = vbar + cbar;
    split_sum(3, 3, sb, wb, bm, bp);
}

static void rpt2_euler(const rp_t *rp, int ixy, const double *ql, const double *qr,
                       const double *asdq, double *bm, double *bp)
{
    const double gamma1 = rp->pd[0] - 1.0;
    const int mu = ixy, mv = 3 - ixy;
    double rhsqrtl = sqrt(ql[0]), rhsqrtr = sqrt(qr[0]);
    double pl = euler_pressure(gamma1, ql);
    double pr = euler_pressure(gamma1, qr);
    double rhsq2 = rhsqrtl + rhsqrtr;
    double u = (ql[mu] / rhsqrtl + qr[mu] / rhsqrtr) / rhsq2;
    double v = (ql[mv] / rhsqrtl + qr[mv] / rhsqrtr) / rhsq2;
    double enth = ((ql[3] + pl) / rhsqrtl + (qr[3] + pr) / rhsqrtr) / rhsq2;
    double u2v2 = u * u + v * v;
    double c2 = gamma1 * (enth - 0.5 * u2v2);
    double a = sqrt(c2);
    double g1a2 = gamma1 / c2;
    double euv = enth - u2v2;
    double a3 = g1a2 * (euv * asdq[0] + u * asdq[mu] + v * asdq[mv] - asdq[3]);
    double a2 = asdq[mu] - u * asdq[0];
    double a4 = (asdq[mv] + (a - v) * asdq[0] - a * a3) / (2.0 * a);
    double a1 = asdq[0] - a3 - a4;
    double wb[16], sb[4];
    wb[0] = a1; wb[mu] = a1 * u; wb[mv] = a1 * (v - a); wb[3] = a1 * (enth - v * a);
    sb[0] = v - a;
    wb[4] = a3; wb[4 + mu] = a3 * u; wb[4 + mv] = a3 * v; wb[7] = a3 * 0.5 * u2v2;
    sb[1] = v;
    wb[8] = 0.0; wb[8 + mu] = a2; wb[8 + mv] = 0.0; wb[11] = a2 * u;
    sb[2] = v;
    wb[12] = a4; wb[12 + mu] = a4 * u; wb[12 + mv] = a4 * (v + a); wb[15] = a4 * (enth + v * a);
    sb[3] = v + a;
    split_sum(4, 4, sb, wb, bm, bp);
}

/* Variable-coefficient acoustics: the fluctuation asdq entering a cell is
 * split into the part transmitted down into the cell below (speed -c_m,
 * eigenvector (-Zm, 0, 1) against the cell's own impedance Z) and the part
 * transmitted up into the cell above (speed +c_p, eigenvector (Zp, 0, 1));
 * reflection at the interfaces is what the two parts do not carry
 * (upstream rpt2_vc_acoustics.f90).  am / a0 / ap: aux of the cells below,
 * at and above the cell that receives asdq. */
static void rpt2_vc_acoustics(int ixy, const double *am, const double *a0, const double *ap,
                              const double *asdq, double *bm, double *bp)
{
    const int mu = ixy, mv = 3 - ixy;
    const double cm = am[1], cp = ap[1];
    const double zm = am[0] * am[1], zz = a0[0] * a0[1], zp = ap[0] * ap[1];
    double a1 = (-asdq[0] + zz * asdq[mv]) / (zm + zz);
    double a2 = (asdq[0] + zz * asdq[mv]) / (zz + zp);
    bm[0] = cm * a1 * zm; bm[mu] = 0.0; bm[mv] = -cm * a1;
    bp[0] = cp * a2 * zp; bp[mu] = 0.0; bp[mv] = cp * a2;
}

/* am / a0 / ap: aux of the cells below / at / above the cell that receives
 * asdq (cell e-1 for amdq, cell e for apdq), for solvers with aux. */
static void rpt2(const rp_t *rp, int ixy, const double *ql, const double *qr,
                 const double *am, const double *a0, const double *ap,
                 const double *asdq, double *bm, double *bp)
{
    switch (rp->id) {
    case RP_ACOUSTICS: rpt2_acoustics(rp, ixy, ql, qr, asdq, bm, bp); return;
    case RP_SHALLOW_ROE_EFIX:
    case RP_SHALLOW_BATHY_FWAVE: rpt2_shallow(rp, ixy, ql, qr, asdq, bm, bp); return;
    case RP_VC_ACOUSTICS: rpt2_vc_acoustics(ixy, am, a0, ap, asdq, bm, bp); return;
    default: rpt2_euler(rp, ixy, ql, qr, asdq, bm, bp); return;
    }
}

/* Wave limiter function phi(theta) (FVMHP sec. 6.12; upstream philim):
 * 1 minmod, 2 superbee, 3 van Leer, 4 monotonized centred (MC). */
static double philim(int id, double r)
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

/* ------------------------------------------------------------------------
 * One 1D slice of n interior cells (cells -2..n+1 present), following
 * flux2: Riemann problems at edges -1..n+1, Godunov fluctuations, CFL,
 * limited second-order correction fluxes, transverse splitting.
 * Edge e lies between cells e-1 and e.  Arrays are indexed with offset 2.
 * Outputs (zeroed here):
 *   qadd[c]  first-order update of cell c (already multiplied by dtdx)
 *   fadd[e]  correction flux at edge e
 *   g1[c], g2[c]  transverse correction fluxes at the low / high
 *                 transverse edge of cell c of this slice
 * ---------------------------------------------------------------------- */
typedef struct {
    double *wave, *s, *amdq, *apdq, *cqxx, *bm, *bp;
} work_t;

static int flux2_slice(const rp_t *rp, int ixy, int n, const double *q1d, double dtdx,
                       int order, int tw, const int *mthlim,
                       double *qadd, double *fadd, double *g1, double *g2, double *cfl1d,
                       const work_t *wk, int maux, const double *auxm, const double *aux0,
                       const double *auxp, const double *kap)
{
    const int m = rp->m, mw = rp->mw;
    const int off = 2;
    int e, k, p, bad = 0;
#define Q(c) (q1d + (size_t)((c) + off) * m)
#define W(e) (wk->wave + (size_t)((e) + off) * mw * m)
#define S(e) (wk->s + (size_t)((e) + off) * mw)
#define AM(e) (wk->amdq + (size_t)((e) + off) * m)
#define AP(e) (wk->apdq + (size_t)((e) + off) * m)
#define CQ(e) (wk->cqxx + (size_t)((e) + off) * m)
#define BM(e) (wk->bm + (size_t)((e) + off) * m)
#define BP(e) (wk->bp + (size_t)((e) + off) * m)
#define A1(arr, c) ((arr) + (size_t)((c) + off) * m)
#define AX(arr, c) ((arr) ? (arr) + (size_t)((c) + off) * maux : NULL)
/* dtdx1d of flux2: dt/dx over the capacity of cell c (kap[c + off]) */
#define DTDX(c) (kap ? dtdx / kap[(c) + off] : dtdx)

    for (e = -1; e <= n + 1; e++)
        bad |= rpn2(rp, ixy, Q(e - 1), Q(e), AX(aux0, e - 1), AX(aux0, e), W(e), S(e), AM(e),
                    AP(e));

    for (e = -2; e <= n + 1; e++)
        for (k = 0; k < m; k++) {
            A1(qadd, e)[k] = 0.0;
            A1(fadd, e)[k] = 0.0;
            A1(g1, e)[k] = 0.0;
            A1(g2, e)[k] = 0.0;
        }

    /* first-order (Godunov) updates */
    for (e = 0; e <= n; e++)
        for (k = 0; k < m; k++) {
            A1(qadd, e)[k] = A1(qadd, e)[k] - DTDX(e) * AP(e)[k];
            A1(qadd, e - 1)[k] = A1(qadd, e - 1)[k] - DTDX(e - 1) * AM(e)[k];
        }

    /* Courant number over the edges of this slice */
    double cfl = 0.0;
    for (e = 0; e <= n; e++)
        for (p = 0; p < mw; p++) {
            double sp = S(e)[p];
            cfl = fmax(cfl, fmax(DTDX(e) * sp, -DTDX(e - 1) * sp));
        }
    *cfl1d = cfl;

    if (order == 2) {
        /* limit each wave family against its upwind neighbour; the neighbour
         * waves used for theta are the unlimited ones */
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
                double phi = philim(mthlim[p], r);
                for (k = 0; k < m; k++) W(e)[p * m + k] = phi * W(e)[p * m + k];
            }
        }
        /* correction flux: |s| (1 - |s| dt/dx) W for waves, sign(s) (1 - |s|
         * dt/dx) Z for f-waves (the f-wave already carries the speed) */
        const int fwave = rp->id == RP_SHALLOW_BATHY_FWAVE;
        for (e = 0; e <= n; e++)
            for (k = 0; k < m; k++) {
                /* dt/dx averaged over the edge's two cells */
                double dtdxave = 0.5 * (DTDX(e - 1) + DTDX(e));
                double c = 0.0;
                for (p = 0; p < mw; p++) {
                    double sa = fabs(S(e)[p]);
                    if (fwave)
                        c = c + copysign(1.0, S(e)[p]) * (1.0 - sa * dtdxave) * W(e)[p * m + k];
                    else
                        c = c + sa * (1.0 - sa * dtdxave) * W(e)[p * m + k];
                }
                CQ(e)[k] = c;
                A1(fadd, e)[k] = A1(fadd, e)[k] + 0.5 * c;
            }
    }

    if (tw > 0) {
        if (order == 2 && tw == 2)
            for (e = 0; e <= n; e++)
                for (k = 0; k < m; k++) {
                    AM(e)[k] = AM(e)[k] + CQ(e)[k];
                    AP(e)[k] = AP(e)[k] - CQ(e)[k];
                }
        /* the half dt/dx of the cell the fluctuation goes into */
        for (e = 0; e <= n; e++)
            rpt2(rp, ixy, Q(e - 1), Q(e), AX(auxm, e - 1), AX(aux0, e - 1), AX(auxp, e - 1),
                 AM(e), BM(e), BP(e));
        for (e = 0; e <= n; e++)
            for (k = 0; k < m; k++) {
                const double h = 0.5 * DTDX(e - 1);
                A1(g1, e - 1)[k] = A1(g1, e - 1)[k] - h * BM(e)[k];
                A1(g2, e - 1)[k] = A1(g2, e - 1)[k] - h * BP(e)[k];
            }
        for (e = 0; e <= n; e++)
            rpt2(rp, ixy, Q(e - 1), Q(e), AX(auxm, e), AX(aux0, e), AX(auxp, e), AP(e), BM(e),
                 BP(e));
        for (e = 0; e <= n; e++)
            for (k = 0; k < m; k++) {
                const double h = 0.5 * DTDX(e);
                A1(g1, e)[k] = A1(g1, e)[k] - h * BM(e)[k];
                A1(g2, e)[k] = A1(g2, e)[k] - h * BP(e)[k];
            }
    }
#undef Q
#undef W
#undef S
#undef AM
#undef AP
#undef CQ
#undef BM
#undef BP
#undef A1
#undef AX
#undef DTDX
    return bad;
}

/* ------------------------------------------------------------------------
 * Exported entry points (ctypes).
 * ---------------------------------------------------------------------- */

int gclaw_ref_shape(int rp_id, int *m, int *mw) { return rp_shape(rp_id, m, mw); }

/* Ghost fill as PyClaw's _apply_bcs does it for a single-process run:
 * x boundaries first over every row (y-ghost rows included), then y
 * boundaries over every column (x-ghost columns included).  extrap copies the
 * edge cell, periodic wraps, wall mirrors and negates the normal
 * momentum/velocity component (component 1 for x, 2 for y).  q is (m,mx,my)
 * Fortran order, qbc is (m,mx+2g,my+2g). */
static int fill_ghosts_impl(int m, int mx, int my, int g, const int *bc_lower,
                            const int *bc_upper, const double *q, double *qbc, int negate);

int gclaw_ref_fill_ghosts(int m, int mx, int my, int g, const int *bc_lower,
                          const int *bc_upper, const double *q, double *qbc)
{
    return fill_ghosts_impl(m, mx, my, g, bc_lower, bc_upper, q, qbc, 1);
}

/* Ghost fill of an aux array (PyClaw's aux_bc_lower / aux_bc_upper): as for
 * q, except that wall boundaries mirror without negating any component. */
int gclaw_ref_fill_aux_ghosts(int maux, int mx, int my, int g, const int *bc_lower,
                              const int *bc_upper, const double *aux, double *auxbc)
{
    return fill_ghosts_impl(maux, mx, my, g, bc_lower, bc_upper, aux, auxbc, 0);
}

static int fill_ghosts_impl(int m, int mx, int my, int g, const int *bc_lower,
                            const int *bc_upper, const double *q, double *qbc, int negate)
{
    if (m < 1 || m > MAXM || mx < g || my < g || g < 1) return ERR_ARG;
    for (int d = 0; d < 2; d++)
        if (bc_lower[d] < BC_EXTRAP || bc_lower[d] > BC_WALL || bc_upper[d] < BC_EXTRAP ||
            bc_upper[d] > BC_WALL)
            return ERR_ARG;
    const int nx = mx + 2 * g, ny = my + 2 * g;
#define QB(k, i, j) qbc[(size_t)(k) + (size_t)m * ((size_t)(i) + (size_t)nx * (size_t)(j))]
    for (int j = 0; j < my; j++)
        for (int i = 0; i < mx; i++)
            for (int k = 0; k < m; k++)
                QB(k, i + g, j + g) = q[(size_t)k + (size_t)m * ((size_t)i + (size_t)mx * j)];
    /* x direction, all rows */
    for (int j = 0; j < ny; j++)
        for (int l = 0; l < g; l++) {
            int src_lo, src_hi, neg_lo = 0, neg_hi = 0;
            switch (bc_lower[0]) {
            case BC_EXTRAP: src_lo = g; break;
            case BC_PERIODIC: src_lo = l + mx; break;
            default: src_lo = 2 * g - 1 - l; neg_lo = negate; break;
            }
            switch (bc_upper[0]) {
            case BC_EXTRAP: src_hi = g + mx - 1; break;
            case BC_PERIODIC: src_hi = g + l; break;
            default: src_hi = g + mx - 1 - l; neg_hi = negate; break;
            }
            for (int k = 0; k < m; k++) {
                double vlo = QB(k, src_lo, j), vhi = QB(k, src_hi, j);
                QB(k, l, j) = (neg_lo && k == 1) ? -vlo : vlo;
                QB(k, g + mx + l, j) = (neg_hi && k == 1) ? -vhi : vhi;
            }
        }
    /* y direction, all columns */
    for (int l = 0; l < g; l++)
        for (int i = 0; i < nx; i++) {
            int src_lo, src_hi, neg_lo = 0, neg_hi = 0;
            switch (bc_lower[1]) {
            case BC_EXTRAP: src_lo = g; break;
            case BC_PERIODIC: src_lo = l + my; break;
            default: src_lo = 2 * g - 1 - l; neg_lo = negate; break;
            }
            switch (bc_upper[1]) {
            case BC_EXTRAP: src_hi = g + my - 1; break;
            case BC_PERIODIC: src_hi = g + l; break;
            default: src_hi = g + my - 1 - l; neg_hi = negate; break;
            }
            for (int k = 0; k < m; k++) {
                double vlo = QB(k, i, src_lo), vhi = QB(k, i, src_hi);
                QB(k, i, l) = (neg_lo && k == 2) ? -vlo : vlo;
                QB(k, i, g + my + l) = (neg_hi && k == 2) ? -vhi : vhi;
            }
        }
#undef QB
    return 0;
}

/* One Riemann problem at an edge, for known-answer tests. */
int gclaw_ref_rpn2(int rp_id, const double *pd, int ixy, const double *ql, const double *qr,
                   double *wave, double *s, double *amdq, double *apdq)
{
    rp_t rp;
    rp.id = rp_id;
    if (rp_shape(rp_id, &rp.m, &rp.mw) || (ixy != 1 && ixy != 2)) return ERR_ARG;
    /* solvers with aux: gclaw_ref_rpn2_aux */
    if (rp_id == RP_VC_ACOUSTICS || rp_id == RP_SHALLOW_BATHY_FWAVE) return ERR_ARG;
    memcpy(rp.pd, pd, sizeof rp.pd);
    return rpn2(&rp, ixy, ql, qr, NULL, NULL, wave, s, amdq, apdq) ? ERR_NONPHYSICAL : 0;
}

/* The same with the aux values of the two cells (solvers with aux). */
int gclaw_ref_rpn2_aux(int rp_id, const double *pd, int ixy, const double *ql,
                       const double *qr, const double *al, const double *ar, double *wave,
                       double *s, double *amdq, double *apdq)
{
    rp_t rp;
    rp.id = rp_id;
    if (rp_shape(rp_id, &rp.m, &rp.mw) || (ixy != 1 && ixy != 2)) return ERR_ARG;
    memcpy(rp.pd, pd, sizeof rp.pd);
    return rpn2(&rp, ixy, ql, qr, al, ar, wave, s, amdq, apdq) ? ERR_NONPHYSICAL : 0;
}

int gclaw_ref_rpt2(int rp_id, const double *pd, int ixy, const double *ql, const double *qr,
                   const double *asdq, double *bm, double *bp)
{
    rp_t rp;
    rp.id = rp_id;
    if (rp_shape(rp_id, &rp.m, &rp.mw) || (ixy != 1 && ixy != 2)) return ERR_ARG;
    if (rp_id == RP_VC_ACOUSTICS) return ERR_ARG; /* needs aux: gclaw_ref_rpt2_aux */
    memcpy(rp.pd, pd, sizeof rp.pd);
    rpt2(&rp, ixy, ql, qr, NULL, NULL, NULL, asdq, bm, bp);
    return 0;
}

/* The same with the aux of the cells below, at and above the receiving cell. */
int gclaw_ref_rpt2_aux(int rp_id, const double *pd, int ixy, const double *am,
                       const double *a0, const double *ap, const double *asdq, double *bm,
                       double *bp)
{
    rp_t rp;
    rp.id = rp_id;
    if (rp_shape(rp_id, &rp.m, &rp.mw) || (ixy != 1 && ixy != 2)) return ERR_ARG;
    memcpy(rp.pd, pd, sizeof rp.pd);
    rpt2(&rp, ixy, NULL, NULL, am, a0, ap, asdq, bm, bp);
    return 0;
}

double gclaw_ref_philim(int id, double r) { return philim(id, r); }

/* The classic unsplit step (step2).  qold and qnew are qbc-shaped
 * (m, mx+2g, my+2g), Fortran order, ghosts of qold filled; g must be 2.
 * qnew receives qold plus all updates (its ghost entries are qold's).
 * pd: problem data (acoustics: rho, bulk, cc, zz; shallow: grav;
 * euler: gamma, efix).  Returns 0, or ERR_NONPHYSICAL if a Riemann problem
 * met a non-physical state. */
static int step2_dirs(int rp_id, const double *pd, int g, int mx, int my, const double *qold,
                      double *qnew, double dx, double dy, double dt, int order, int tw,
                      const int *mthlim, double *cfl_out, int nthreads, int ixy_lo,
                      int ixy_hi, int maux, const double *auxbc, int mcapa);

int gclaw_ref_step2(int rp_id, const double *pd, int g, int mx, int my, const double *qold,
                    double *qnew, double dx, double dy, double dt, int order, int tw,
                    const int *mthlim, double *cfl_out, int nthreads)
{
    /* solvers with aux: gclaw_ref_step2_aux */
    if (rp_id == RP_VC_ACOUSTICS || rp_id == RP_SHALLOW_BATHY_FWAVE) return ERR_ARG;
    return step2_dirs(rp_id, pd, g, mx, my, qold, qnew, dx, dy, dt, order, tw, mthlim, cfl_out,
                      nthreads, 1, 2, 0, NULL, 0);
}

/* step2 with an aux array: auxbc is (maux, mx+2g, my+2g), Fortran order,
 * ghosts filled (gclaw_ref_fill_aux_ghosts).  mcapa: 1-based index of the
 * capacity field in aux (classic2's mcapa, PyClaw state.index_capa + 1), 0
 * for none; with a capacity kappa the step is the capacity-form update of
 * LeVeque 1997 sec. 5 / FVMHP sec. 6.16: dt/dx becomes dt/(kappa dx) per
 * cell (fluctuations, Courant numbers, transverse terms, and the average of
 * the edge's two cells in the correction flux), and the flux differences of
 * cell (i,j) are divided by its kappa. */
int gclaw_ref_step2_aux(int rp_id, const double *pd, int g, int mx, int my, const double *qold,
                        double *qnew, int maux, const double *auxbc, double dx, double dy,
                        double dt, int order, int tw, const int *mthlim, double *cfl_out,
                        int nthreads, int mcapa)
{
    if (maux < 1 || maux > MAXM || !auxbc || mcapa < 0 || mcapa > maux) return ERR_ARG;
    return step2_dirs(rp_id, pd, g, mx, my, qold, qnew, dx, dy, dt, order, tw, mthlim, cfl_out,
                      nthreads, 1, 2, maux, auxbc, mcapa);
}

/* One sweep of PyClaw's dimensionally split step (classic2 step2ds,
 * upstream pyclaw/src/pyclaw/classic/step2ds.f90): the slices of direction
 * ixy only, without transverse propagation, from the ghost-filled qold into
 * qnew (same shapes as step2).  *cfl_out is that sweep's Courant number. */
int gclaw_ref_step2ds(int rp_id, const double *pd, int g, int mx, int my, const double *qold,
                      double *qnew, double dx, double dy, double dt, int order,
                      const int *mthlim, int ixy, double *cfl_out, int nthreads)
{
    if (ixy != 1 && ixy != 2) return ERR_ARG;
    if (rp_id == RP_VC_ACOUSTICS || rp_id == RP_SHALLOW_BATHY_FWAVE) return ERR_ARG;
    return step2_dirs(rp_id, pd, g, mx, my, qold, qnew, dx, dy, dt, order, 0, mthlim, cfl_out,
                      nthreads, ixy, ixy, 0, NULL, 0);
}

static int step2_dirs(int rp_id, const double *pd, int g, int mx, int my, const double *qold,
                      double *qnew, double dx, double dy, double dt, int order, int tw,
                      const int *mthlim, double *cfl_out, int nthreads, int ixy_lo, int ixy_hi,
                      int maux, const double *auxbc, int mcapa)
{
    rp_t rp;
    rp.id = rp_id;
    if (rp_shape(rp_id, &rp.m, &rp.mw) || g != 2 || mx < 2 || my < 2) return ERR_ARG;
    if (order < 1 || order > 2 || tw < 0 || tw > 2) return ERR_ARG;
    memcpy(rp.pd, pd, sizeof rp.pd);
    const int m = rp.m, mw = rp.mw;
    const int nx = mx + 2 * g, ny = my + 2 * g;
    const double dtdx = dt / dx, dtdy = dt / dy;
    const size_t qsize = (size_t)m * nx * ny;
    memcpy(qnew, qold, qsize * sizeof(double));

    /* per-slice outputs: [slice][cell(+2 offset)][k] */
    const int nmax = (mx > my ? mx : my) + 4;
    const int nslx = my + 2, nsly = mx + 2;
    const int nsl = nslx > nsly ? nslx : nsly;
    const size_t per = (size_t)nmax * m;
    double *QA = malloc(sizeof(double) * per * nsl);
    double *FA = malloc(sizeof(double) * per * nsl);
    double *G1 = malloc(sizeof(double) * per * nsl);
    double *G2 = malloc(sizeof(double) * per * nsl);
    double *cfls = malloc(sizeof(double) * nsl);
    if (!QA || !FA || !G1 || !G2 || !cfls) {
        free(QA); free(FA); free(G1); free(G2); free(cfls);
        return ERR_ALLOC;
    }
    if (nthreads < 1) nthreads = 1;
    int bad = 0;
    double cfl = 0.0;

    for (int ixy = ixy_lo; ixy <= ixy_hi; ixy++) {
        const int n = (ixy == 1) ? mx : my;
        const int ns = (ixy == 1) ? nslx : nsly;
        const double dtdn = (ixy == 1) ? dtdx : dtdy;
#pragma omp parallel num_threads(nthreads) reduction(| : bad)
        {
            work_t wk;
            double *q1d = malloc(sizeof(double) * per);
            wk.wave = malloc(sizeof(double) * (size_t)nmax * mw * m);
            wk.s = malloc(sizeof(double) * (size_t)nmax * mw);
            wk.amdq = malloc(sizeof(double) * per);
            wk.apdq = malloc(sizeof(double) * per);
            wk.cqxx = malloc(sizeof(double) * per);
            wk.bm = malloc(sizeof(double) * per);
            wk.bp = malloc(sizeof(double) * per);
            /* aux of the slice and of the slices below and above it, and the
             * slice's capacities */
            double *a1d[3] = {NULL, NULL, NULL};
            if (maux)
                for (int d = 0; d < 3; d++) a1d[d] = malloc(sizeof(double) * (size_t)nmax * maux);
            double *k1d = mcapa ? malloc(sizeof(double) * (size_t)nmax) : NULL;
#pragma omp for schedule(static)
            for (int sl = 0; sl < ns; sl++) {
                /* slice index sl -> row j = sl-1 (x-sweep) or column i = sl-1 */
                for (int c = -2; c < n + 2; c++)
                    for (int k = 0; k < m; k++) {
                        size_t src = (ixy == 1)
                                         ? (size_t)k + (size_t)m * ((size_t)(c + g) + (size_t)nx * (sl - 1 + g))
                                         : (size_t)k + (size_t)m * ((size_t)(sl - 1 + g) + (size_t)nx * (c + g));
                        q1d[(size_t)(c + 2) * m + k] = qold[src];
                    }
                for (int d = 0; d < 3 && maux; d++) {
                    const int t = sl - 2 + d; /* transverse index of slice sl-1+d-1 */
                    for (int c = -2; c < n + 2; c++)
                        for (int k = 0; k < maux; k++) {
                            size_t src = (ixy == 1)
                                             ? (size_t)k + (size_t)maux * ((size_t)(c + g) + (size_t)nx * (t + g))
                                             : (size_t)k + (size_t)maux * ((size_t)(t + g) + (size_t)nx * (c + g));
                            a1d[d][(size_t)(c + 2) * maux + k] = auxbc[src];
                        }
                }
                if (mcapa)
                    for (int c = -2; c < n + 2; c++) k1d[c + 2] = a1d[1][(size_t)(c + 2) * maux + mcapa - 1];
                bad |= flux2_slice(&rp, ixy, n, q1d, dtdn, order, tw, mthlim, QA + per * sl,
                                   FA + per * sl, G1 + per * sl, G2 + per * sl, &cfls[sl], &wk,
                                   maux, a1d[0], a1d[1], a1d[2], k1d);
            }
            for (int d = 0; d < 3; d++) free(a1d[d]);
            free(k1d);
            free(q1d); free(wk.wave); free(wk.s); free(wk.amdq); free(wk.apdq);
            free(wk.cqxx); free(wk.bm); free(wk.bp);
        }
        for (int sl = 0; sl < ns; sl++) cfl = fmax(cfl, cfls[sl]);

        /* ordered accumulation: for cell (i,j) the slice before, the own slice,
         * the slice after */
        const double dtdt = (ixy == 1) ? dtdy : dtdx; /* transverse dt/d */
        const int nt = (ixy == 1) ? my : mx;         /* number of slices' interior */
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int t = 0; t < nt; t++) {
            const int sl = t + 1; /* slice of interior index t */
            for (int c = 0; c < n; c++) {
                size_t dst = (ixy == 1) ? (size_t)m * ((size_t)(c + g) + (size_t)nx * (t + g))
                                        : (size_t)m * ((size_t)(t + g) + (size_t)nx * (c + g));
                const double *g2prev = G2 + per * (sl - 1) + (size_t)(c + 2) * m;
                const double *g1next = G1 + per * (sl + 1) + (size_t)(c + 2) * m;
                const double *qa = QA + per * sl + (size_t)(c + 2) * m;
                const double *fa0 = FA + per * sl + (size_t)(c + 2) * m;
                const double *fa1 = fa0 + m;
                const double *g1o = G1 + per * sl + (size_t)(c + 2) * m;
                const double *g2o = G2 + per * sl + (size_t)(c + 2) * m;
                if (mcapa) {
                    /* the flux differences and transverse terms over the
                     * capacity of this cell */
                    const double kc = auxbc[(size_t)(mcapa - 1) + (size_t)maux * (dst / m)];
                    for (int k = 0; k < m; k++) {
                        double v = qnew[dst + k];
                        v = v + dtdt * g2prev[k] / kc;
                        v = v + qa[k] - (dtdn * (fa1[k] - fa0[k]) + dtdt * (g2o[k] - g1o[k])) / kc;
                        v = v - dtdt * g1next[k] / kc;
                        qnew[dst + k] = v;
                    }
                    continue;
                }
                for (int k = 0; k < m; k++) {
                    double v = qnew[dst + k];
                    v = v + dtdt * g2prev[k];
                    v = v + qa[k] - dtdn * (fa1[k] - fa0[k]) - dtdt * (g2o[k] - g1o[k]);
                    v = v - dtdt * g1next[k];
                    qnew[dst + k] = v;
                }
            }
        }
    }
    free(QA); free(FA); free(G1); free(G2); free(cfls);
    *cfl_out = cfl;
    return bad ? ERR_NONPHYSICAL : 0;
}

/* Convenience: ghost fill + step on interior-shaped arrays (m, mx, my). */
int gclaw_ref_step(int rp_id, const double *pd, int mx, int my, const double *q, double *qout,
                   double dx, double dy, double dt, int order, int tw, const int *mthlim,
                   const int *bc_lower, const int *bc_upper, double *cfl_out, int nthreads)
{
    int m, mw;
    if (rp_shape(rp_id, &m, &mw)) return ERR_ARG;
    const int g = 2, nx = mx + 4, ny = my + 4;
    size_t nb = (size_t)m * nx * ny;
    double *qa = malloc(sizeof(double) * nb), *qb = malloc(sizeof(double) * nb);
    if (!qa || !qb) {
        free(qa); free(qb);
        return ERR_ALLOC;
    }
    int rc = gclaw_ref_fill_ghosts(m, mx, my, g, bc_lower, bc_upper, q, qa);
    if (rc == 0)
        rc = gclaw_ref_step2(rp_id, pd, g, mx, my, qa, qb, dx, dy, dt, order, tw, mthlim, cfl_out,
                             nthreads);
    if (rc == 0 || rc == ERR_NONPHYSICAL)
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++)
                for (int k = 0; k < m; k++)
                    qout[(size_t)k + (size_t)m * ((size_t)i + (size_t)mx * j)] =
                        qb[(size_t)k + (size_t)m * ((size_t)(i + g) + (size_t)nx * (j + g))];
    free(qa);
    free(qb);
    return rc;
}

/* PyClaw's dimensionally split step (Godunov splitting, ClawSolver2D with
 * dimensional_split=True, upstream pyclaw/src/pyclaw/classic/solver.py):
 * boundary conditions, the x-sweep, boundary conditions again on its
 * result, the y-sweep; *cfl_out = max of the two sweeps' Courant numbers.
 * Interior-shaped arrays (m, mx, my). */
int gclaw_ref_step_split(int rp_id, const double *pd, int mx, int my, const double *q,
                         double *qout, double dx, double dy, double dt, int order,
                         const int *mthlim, const int *bc_lower, const int *bc_upper,
                         double *cfl_out, int nthreads)
{
    int m, mw;
    if (rp_shape(rp_id, &m, &mw)) return ERR_ARG;
    const int g = 2, nx = mx + 4, ny = my + 4;
    size_t nb = (size_t)m * nx * ny;
    double *qa = malloc(sizeof(double) * nb), *qb = malloc(sizeof(double) * nb);
    double *qi = malloc(sizeof(double) * (size_t)m * mx * my);
    if (!qa || !qb || !qi) {
        free(qa); free(qb); free(qi);
        return ERR_ALLOC;
    }
    double cfl[2] = {0.0, 0.0};
    int rc = 0, bad = 0;
    const double *src = q;
    for (int ixy = 1; ixy <= 2 && (rc == 0 || rc == ERR_NONPHYSICAL); ixy++) {
        rc = gclaw_ref_fill_ghosts(m, mx, my, g, bc_lower, bc_upper, src, qa);
        if (rc) break;
        rc = gclaw_ref_step2ds(rp_id, pd, g, mx, my, qa, qb, dx, dy, dt, order, mthlim, ixy,
                               &cfl[ixy - 1], nthreads);
        if (rc == ERR_NONPHYSICAL) bad = 1;
        double *dst = (ixy == 1) ? qi : qout;
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++)
                for (int k = 0; k < m; k++)
                    dst[(size_t)k + (size_t)m * ((size_t)i + (size_t)mx * j)] =
                        qb[(size_t)k + (size_t)m * ((size_t)(i + g) + (size_t)nx * (j + g))];
        src = qi;
    }
    free(qa); free(qb); free(qi);
    *cfl_out = cfl[0] > cfl[1] ? cfl[0] : cfl[1];
    if (rc && rc != ERR_NONPHYSICAL) return rc;
    return bad ? ERR_NONPHYSICAL : 0;
}

/* Ghost fill of q and aux + step2 on interior-shaped arrays, for solvers
 * with an aux array (m, mx, my) / (maux, mx, my). */
int gclaw_ref_step_aux(int rp_id, const double *pd, int mx, int my, const double *q,
                       double *qout, int maux, const double *aux, double dx, double dy,
                       double dt, int order, int tw, const int *mthlim, const int *bc_lower,
                       const int *bc_upper, const int *aux_bc_lower, const int *aux_bc_upper,
                       double *cfl_out, int nthreads, int mcapa)
{
    int m, mw;
    if (rp_shape(rp_id, &m, &mw) || maux < 1 || maux > MAXM) return ERR_ARG;
    const int g = 2, nx = mx + 4, ny = my + 4;
    size_t nb = (size_t)m * nx * ny;
    double *qa = malloc(sizeof(double) * nb), *qb = malloc(sizeof(double) * nb);
    double *ab = malloc(sizeof(double) * (size_t)maux * nx * ny);
    if (!qa || !qb || !ab) {
        free(qa); free(qb); free(ab);
        return ERR_ALLOC;
    }
    int rc = gclaw_ref_fill_ghosts(m, mx, my, g, bc_lower, bc_upper, q, qa);
    if (rc == 0) rc = gclaw_ref_fill_aux_ghosts(maux, mx, my, g, aux_bc_lower, aux_bc_upper, aux, ab);
    if (rc == 0)
        rc = gclaw_ref_step2_aux(rp_id, pd, g, mx, my, qa, qb, maux, ab, dx, dy, dt, order, tw,
                                 mthlim, cfl_out, nthreads, mcapa);
    if (rc == 0 || rc == ERR_NONPHYSICAL)
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++)
                for (int k = 0; k < m; k++)
                    qout[(size_t)k + (size_t)m * ((size_t)i + (size_t)mx * j)] =
                        qb[(size_t)k + (size_t)m * ((size_t)(i + g) + (size_t)nx * (j + g))];
    free(qa); free(qb); free(ab);
    return rc;
}
