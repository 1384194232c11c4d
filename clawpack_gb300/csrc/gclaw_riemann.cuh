// gclaw_riemann.cuh -- device Riemann solvers and wave limiters for the
// classic unsplit 2D step.
//
// Normal solvers (rpn2) and transverse solvers (rpt2) of the clawpack.riemann
// modules acoustics_2D, shallow_roe_with_efix_2D and euler_4wave_2D
// (upstream riemann/src/rpn2_acoustics.f90, rpt2_acoustics.f90,
// rpn2_shallow_roe_with_efix.f90, rpt2_shallow_roe_with_efix.f90,
// rpn2_euler_4wave.f90, rpt2_euler.f90; the riemann submodule is empty in the
// mounted clawpack 5.14.0 tree, meson.build:65).  The mathematics is that of
// LeVeque, Finite Volume Methods for Hyperbolic Problems (2002): Roe
// linearisations (sec. 15.3), the Harten-Hyman entropy fix (sec. 15.3.5),
// transverse splitting with the transverse eigenstructure at the edge's Roe
// state (ch. 21), wave limiters (sec. 6.12).
//
// Every expression is written in the operation order of the CPU oracle so
// that an FP64 build without multiply-add contraction reproduces it bit for
// bit.  Differences from the reference's per-edge code are layout only: the
// Roe state of an edge is computed once by rpn2 and handed to rpt2 (rpt2
// recomputes the identical expressions upstream), and ixy is a template
// parameter.
//
// Conventions: ql is the cell left of (below) the edge, qr the cell right of
// (above) it.  W is [MW][M] row-major, s is [MW].  mu = IXY is the normal
// momentum/velocity component, mv = 3 - IXY the transverse one.
//
// Per-cell quantities that every edge of a cell needs (square roots and
// quotients of the cell state) are computed once per cell by cell_aux into
// NA values and passed to rpn2 as al / ar; each is the same expression the
// per-edge code evaluates, so the results are unchanged bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace gclaw {

// |a|, sqrt(a), 1/sqrt(a) in the type of a: the float forms by their float
// names, so that no float operand is widened to a double call.
template <typename T>
__device__ __forceinline__ T tabs(T a) { return fabs(a); }
template <>
__device__ __forceinline__ float tabs<float>(float a) { return fabsf(a); }
template <typename T>
__device__ __forceinline__ T tsqrt(T a) { return sqrt(a); }
template <>
__device__ __forceinline__ float tsqrt<float>(float a) { return sqrtf(a); }
template <typename T>
__device__ __forceinline__ T trsqrt(T a) { return rsqrt(a); }
template <>
__device__ __forceinline__ float trsqrt<float>(float a) { return rsqrtf(a); }
template <typename T>
__device__ __forceinline__ T tmin(T a, T b) { return fmin(a, b); }
template <typename T>
__device__ __forceinline__ T tmax(T a, T b) { return fmax(a, b); }
template <>
__device__ __forceinline__ float tmin<float>(float a, float b) { return fminf(a, b); }
template <>
__device__ __forceinline__ float tmax<float>(float a, float b) { return fmaxf(a, b); }

// Tests of a value against zero with IEEE results (NaN compares false,
// -0 == +0), and min / max of values known to be in [+0, +inf].  For
// doubles they are integer tests on the bit pattern: GB300 executes FP64
// comparisons, min and max on its FP64 pipe, which is the unit the FP64
// step is bound by, while the integer pipes are idle.
template <typename T>
__device__ __forceinline__ bool gt0(T x) { return x > (T)0; }
template <typename T>
__device__ __forceinline__ bool lt0(T x) { return x < (T)0; }
template <typename T>
__device__ __forceinline__ bool isnan_v(T x) { return x != x; }
template <typename T>
__device__ __forceinline__ T nnmin(T a, T b) { return tmin(a, b); }
template <typename T>
__device__ __forceinline__ T nnmax(T a, T b) { return tmax(a, b); }

constexpr long long F64_INF_BITS = 0x7FF0000000000000LL;
constexpr long long F64_ABS_MASK = 0x7FFFFFFFFFFFFFFFLL;
template <>
__device__ __forceinline__ bool gt0<double>(double x) {
    const long long b = __double_as_longlong(x);
    return b > 0 && b <= F64_INF_BITS;  // sign clear, not +0, not NaN
}
template <>
__device__ __forceinline__ bool lt0<double>(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned long long m = (unsigned long long)(b & F64_ABS_MASK);
    return b < 0 && m - 1ull < (unsigned long long)F64_INF_BITS;  // sign set, 0 < |x| <= inf
}
template <>
__device__ __forceinline__ bool isnan_v<double>(double x) {
    return (__double_as_longlong(x) & F64_ABS_MASK) > F64_INF_BITS;
}
template <>
__device__ __forceinline__ double nnmin<double>(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x < y ? x : y);
}
template <>
__device__ __forceinline__ double nnmax<double>(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x > y ? x : y);
}
// a < b and a >= b (IEEE) when b is in [+0, +inf] and a is >= +0, -0 or NaN
template <typename T>
__device__ __forceinline__ bool nn_lt(T a, T b) { return a < b; }
template <typename T>
__device__ __forceinline__ bool nn_ge(T a, T b) { return a >= b; }
template <>
__device__ __forceinline__ bool nn_lt<double>(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return y <= F64_INF_BITS && x < y;
}
template <>
__device__ __forceinline__ bool nn_ge<double>(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return x <= F64_INF_BITS && x >= y;
}
template <typename T>
__device__ __forceinline__ bool ge0(T x) { return !lt0(x) && !isnan_v(x); }
template <typename T>
__device__ __forceinline__ bool eq0(T x) { return x == (T)0; }
template <>
__device__ __forceinline__ bool eq0<double>(double x) {
    return (__double_as_longlong(x) & F64_ABS_MASK) == 0;
}
template <typename T>
__device__ __forceinline__ bool le0(T x) { return !gt0(x) && !isnan_v(x); }
// min(x, 0) and max(x, 0) as fmin / fmax give them (NaN -> 0), by sign
template <typename T>
__device__ __forceinline__ T neg_part(T x) { return lt0(x) ? x : (T)0; }
template <typename T>
__device__ __forceinline__ T pos_part(T x) { return gt0(x) ? x : (T)0; }

// Running max of |s| over non-NaN speeds, as fmax(m, fabs(s)) gives it.
template <typename T>
__device__ __forceinline__ T max_abs(T m, T s) { return tmax(m, tabs(s)); }
template <>
__device__ __forceinline__ double max_abs<double>(double m, double s) {
    const long long a = __double_as_longlong(s) & F64_ABS_MASK;
    const long long b = __double_as_longlong(m);
    return a <= F64_INF_BITS && a > b ? __longlong_as_double(a) : m;
}

// Reciprocal for the product build.  T = float: the division (approximate
// under -prec-div=false).  T = double: Newton-Raphson iteration for 1/a
// (r <- r + r (1 - a r), quadratic convergence; J.-M. Muller et al.,
// Handbook of Floating-Point Arithmetic, 2nd ed., sec. 4.7) from a seed
// built on the integer and FP32 pipes: the mantissa of a, truncated to a
// float in [1, 2), its FP32 reciprocal, and the exponent of a subtracted
// with an integer add.  The seed is within 2^-22 of 1/a, so two iterations
// (four FP64 fused multiply-adds) reach the last bit or two of the double;
// GB300 executes FP64 arithmetic at 1/64 of its FP32 rate, and the IEEE
// division costs several more FP64 instructions.  Non-positive, denormal,
// infinite, NaN and very large a (exponent field 0, >= 2045) take the
// IEEE division.
template <typename T>
__device__ __forceinline__ T rcp_fast(T a) { return (T)1 / a; }
static __device__ __noinline__ double rcp_slow(double a) { return 1.0 / a; }
template <>
__device__ __forceinline__ double rcp_fast<double>(double a) {
    const long long b = __double_as_longlong(a);
    const int e = (int)((b >> 52) & 0x7ff);  // biased exponent
    if (b <= 0 || e == 0 || e >= 2045) return rcp_slow(a);
    const float mf = __int_as_float(0x3f800000 | (int)((b >> 29) & 0x7fffff));  // in [1, 2)
    const float rf = __frcp_rn(mf);                                             // in (0.5, 1]
    const unsigned u = __float_as_uint(rf);
    // rf as a double, with the exponent of a taken off: 2^(1023 - e) / m
    const long long rb = ((long long)((u >> 23) + 896 + 1023 - e) << 52) |
                         ((long long)(u & 0x7fffff) << 29);
    double r = __longlong_as_double(rb);
    double t = fma(-a, r, 1.0);
    r = fma(r, t, r);
    t = fma(-a, r, 1.0);
    return fma(r, t, r);
}

// a / b: the division in GCLAW_STRICT and FP32, a times the Newton-Raphson
// reciprocal of b for FP64 in the product build (repeated divisors share
// one reciprocal after inlining).
template <typename T>
__device__ __forceinline__ T qdiv(T a, T b) {
#ifdef GCLAW_STRICT
    return a / b;
#else
    if constexpr (sizeof(T) == 8) return a * rcp_fast(b);
    else return a / b;
#endif
}

// copysign(1, s) * x, exactly, as a sign-bit exchange on the integer pipes.
template <typename T>
__device__ __forceinline__ T sign_times(T x, T s);
template <>
__device__ __forceinline__ double sign_times<double>(double x, double s) {
    return __longlong_as_double(__double_as_longlong(x) ^
                                (__double_as_longlong(s) & (long long)0x8000000000000000ull));
}
template <>
__device__ __forceinline__ float sign_times<float>(float x, float s) {
    return __int_as_float(__float_as_int(x) ^ (__float_as_int(s) & (int)0x80000000u));
}

// True when fl(m / h - sqrt(g h)) > 0 cannot hold, decided without the
// division and the square root: h > 0 and either m <= 0 (the quotient is
// not positive) or m^2 < 0.81 g h^3 (|m / h| < 0.9 sqrt(g h) exactly, a
// margin no rounding of either side can close).  A normal-range bound on the
// right side keeps underflow and flush-to-zero out of the test; NaN and
// infinite inputs fall through to the exact evaluation.  Used to skip the
// intermediate-state speeds of the entropy fix when the transonic test is
// certain to fail (every subsonic edge), with unchanged branch decisions.
template <typename T>
__device__ __forceinline__ bool no_right_sonic_point(T h, T m, T g) {
    if (!gt0(h)) return false;
    if (le0(m)) return true;
    const T rhs = (T)0.81 * g * h * h * h;
    const T tiny = sizeof(T) == 8 ? (T)1e-290 : (T)1e-30;
    return nn_ge(rhs, tiny) && nn_lt(m * m, rhs);
}

// ---------------------------------------------------------------------------
// Constant-coefficient acoustics: q = (p, u, v); speeds -c, +c.
// ---------------------------------------------------------------------------
template <typename T>
struct RpAcoustics {
    static constexpr int M = 3, MW = 2, NR = 0, NA = 0, NUA = 0;
    static constexpr bool TNB = false;  // rpn2 does not read the transverse neighbours
    static constexpr bool FWAVE = false, CAPA = false;
    struct Params {
        T cc, zz;
    };
    static Params make(const double *pd) { return Params{(T)pd[2], (T)pd[3]}; }

    __device__ __forceinline__ static void cell_aux(const Params &P, const T *q, T *aux) {}

    // components of wave p that can be nonzero in direction IXY
    template <int IXY>
    __host__ __device__ static constexpr bool wnz(int p, int k) { return k != 3 - IXY; }

    template <int IXY>
    __device__ __forceinline__ static bool rpn2(const Params &P, const T *ql, const T *qr,
                                                const T *al, const T *ar, T *W, T *s, T *am,
                                                T *ap, T *R) {
        constexpr int mu = IXY, mv = 3 - IXY;
        T d0 = qr[0] - ql[0];
        T d1 = qr[mu] - ql[mu];
        T a1 = (-d0 + P.zz * d1) / ((T)2 * P.zz);
        T a2 = (d0 + P.zz * d1) / ((T)2 * P.zz);
        W[0] = -a1 * P.zz; W[mu] = a1; W[mv] = (T)0;
        s[0] = -P.cc;
        W[3] = a2 * P.zz; W[3 + mu] = a2; W[3 + mv] = (T)0;
        s[1] = P.cc;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            am[k] = s[0] * W[k];
            ap[k] = s[1] * W[3 + k];
        }
        return false;
    }

    template <int IXY>
    __device__ __forceinline__ static void rpt2(const Params &P, const T *R, const T *asdq, T *bm,
                                                T *bp) {
        constexpr int mu = IXY, mv = 3 - IXY;
        T a1 = (-asdq[0] + P.zz * asdq[mv]) / ((T)2 * P.zz);
        T a2 = (asdq[0] + P.zz * asdq[mv]) / ((T)2 * P.zz);
        bm[0] = P.cc * a1 * P.zz; bm[mu] = (T)0; bm[mv] = -P.cc * a1;
        bp[0] = P.cc * a2 * P.zz; bp[mu] = (T)0; bp[mv] = P.cc * a2;
    }
};

// ---------------------------------------------------------------------------
// Variable-coefficient acoustics (upstream riemann/src/rpn2_vc_acoustics.f90,
// rpt2_vc_acoustics.f90): q = (p, u, v), a user aux array (rho, c) per cell,
// loaded into the per-cell aux area and turned into (Z = rho c, c) there.
// rpn2 solves the interface problem between impedances Zl and Zr (speeds
// -c_l, +c_r); rpt2 transmits a fluctuation into the cells below and above
// the receiving cell with their speeds and impedances, so rpn2 also reads
// the aux of the cells below and above both edge cells (TNB) and keeps them
// in the edge record R = (c_m, Z_m, Z, c_p, Z_p) of the left cell, then of
// the right cell.  With equal coefficients every expression equals
// RpAcoustics' (bit for bit with -fmad=false).
// ---------------------------------------------------------------------------
template <typename T>
struct RpVcAcoustics {
    static constexpr int M = 3, MW = 2, NR = 10, NA = 2, NUA = 2;
    static constexpr bool TNB = true, FWAVE = false, CAPA = false;
    struct Params {
        int unused;
    };
    static Params make(const double *) { return Params{0}; }

    template <int IXY>
    __host__ __device__ static constexpr bool wnz(int p, int k) { return k != 3 - IXY; }

    // aux holds the cell's (rho, c) on entry and (Z, c) on return
    __device__ __forceinline__ static void cell_aux_user(const Params &, const T *, T *aux) {
        aux[0] = aux[0] * aux[1];
    }

    // al / ar: (Z, c) of the edge cells; bl, tl / br, tr: of the cells below
    // and above the left / right cell in the transverse direction
    template <int IXY>
    __device__ __forceinline__ static bool rpn2_nb(const Params &, const T *ql, const T *qr,
                                                   const T *al, const T *ar, const T *bl,
                                                   const T *tl, const T *br, const T *tr, T *W,
                                                   T *s, T *am, T *ap, T *R) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T d0 = qr[0] - ql[0];
        const T d1 = qr[mu] - ql[mu];
        const T zl = al[0], zr = ar[0];
        const T a1 = (-d0 + zr * d1) / (zl + zr);
        const T a2 = (d0 + zl * d1) / (zl + zr);
        W[0] = -a1 * zl; W[mu] = a1; W[mv] = (T)0;
        s[0] = -al[1];
        W[3] = a2 * zr; W[3 + mu] = a2; W[3 + mv] = (T)0;
        s[1] = ar[1];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            am[k] = s[0] * W[k];
            ap[k] = s[1] * W[3 + k];
        }
        R[0] = bl[1]; R[1] = bl[0]; R[2] = zl; R[3] = tl[1]; R[4] = tl[0];
        R[5] = br[1]; R[6] = br[0]; R[7] = zr; R[8] = tr[1]; R[9] = tr[0];
        return false;
    }

    // SIDE 0: asdq = amdq into the left cell; SIDE 1: apdq into the right cell
    template <int IXY, int SIDE>
    __device__ __forceinline__ static void rpt2s(const Params &, const T *R, const T *asdq, T *bm,
                                                 T *bp) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T *r = R + 5 * SIDE;
        const T cm = r[0], zm = r[1], zz = r[2], cp = r[3], zp = r[4];
        const T a1 = (-asdq[0] + zz * asdq[mv]) / (zm + zz);
        const T a2 = (asdq[0] + zz * asdq[mv]) / (zz + zp);
        bm[0] = cm * a1 * zm; bm[mu] = (T)0; bm[mv] = -cm * a1;
        bp[0] = cp * a2 * zp; bp[mu] = (T)0; bp[mv] = cp * a2;
    }
};

// Sum of min(sb,0) Wb and max(sb,0) Wb over the transverse waves.
template <typename T, int M, int MW>
__device__ __forceinline__ void split_sum(const T *sb, const T *wb, T *bm, T *bp) {
#pragma unroll
    for (int k = 0; k < M; k++) {
        T lo = (T)0, hi = (T)0;
#pragma unroll
        for (int p = 0; p < MW; p++) {
            lo = lo + neg_part(sb[p]) * wb[M * p + k];
            hi = hi + pos_part(sb[p]) * wb[M * p + k];
        }
        bm[k] = lo;
        bp[k] = hi;
    }
}

// ---------------------------------------------------------------------------
// Shallow water, Roe solver with Harten-Hyman entropy fix: q = (h, hu, hv).
// Roe state kept for rpt2: R = (ubar, vbar, cbar).
// ---------------------------------------------------------------------------
template <typename T>
struct RpShallow {
    static constexpr int M = 3, MW = 3, NR = 4, NA = 6, NUA = 0;
    static constexpr bool TNB = false, FWAVE = false, CAPA = false;
    struct Params {
        T g;
        double gd;
        T sg;  // sqrt(g)
    };
    static Params make(const double *pd) { return Params{(T)pd[0], pd[0], (T)sqrt(pd[0])}; }

    // the shear wave carries only the transverse momentum
    template <int IXY>
    __host__ __device__ static constexpr bool wnz(int p, int k) { return p != 1 || k == 3 - IXY; }

    // aux = (sqrt h, hu / sqrt h, hv / sqrt h, hu / h, hv / h, sqrt(g h)).
    // GCLAW_STRICT evaluates each as written; otherwise one square root and
    // one reciprocal per cell (hu / sqrt h = (hu / h) sqrt h, sqrt(g h) =
    // sqrt(g) sqrt h), within two roundings of the quotients.
    __device__ __forceinline__ static void cell_aux(const Params &P, const T *q, T *aux) {
        const T hs = tsqrt(q[0]);
        aux[0] = hs;
#ifdef GCLAW_STRICT
        aux[1] = q[1] / hs;
        aux[2] = q[2] / hs;
        aux[3] = q[1] / q[0];
        aux[4] = q[2] / q[0];
        aux[5] = tsqrt(P.g * q[0]);
#else
        const T rh = rcp_fast(q[0]);
        aux[3] = q[1] * rh;
        aux[4] = q[2] * rh;
        aux[1] = aux[3] * hs;
        aux[2] = aux[4] * hs;
        aux[5] = P.sg * hs;
#endif
    }

    // Roe state R = (ubar, vbar, cbar, 0.5 / cbar).  In FP32-bulk mode,
    // depths below 1e-3 take the square roots and quotients in FP64
    // (near-dry states).
    template <int IXY>
    __device__ __forceinline__ static void roe(const Params &P, const T *ql, const T *qr,
                                               const T *al, const T *ar, T *R) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T hl = ql[0], hr = qr[0];
        T u, v, c;
        if (sizeof(T) == 4 && (hl < (T)1e-3 || hr < (T)1e-3)) {
            double sl = sqrt((double)hl), sr = sqrt((double)hr), s2 = sl + sr;
            u = (T)(((double)ql[mu] / sl + (double)qr[mu] / sr) / s2);
            v = (T)(((double)ql[mv] / sl + (double)qr[mv] / sr) / s2);
            c = (T)sqrt(P.gd * (((double)hl + (double)hr) * 0.5));
        } else {
            const T hsq2 = al[0] + ar[0];
            const T hbar = (hl + hr) * (T)0.5;
#ifdef GCLAW_STRICT
            u = (al[mu] + ar[mu]) / hsq2;
            v = (al[mv] + ar[mv]) / hsq2;
            c = tsqrt(P.g * hbar);
#else
            // one reciprocal for both averages; c and 0.5 / c from one rsqrt
            const T ri = rcp_fast(hsq2);
            u = (al[mu] + ar[mu]) * ri;
            v = (al[mv] + ar[mv]) * ri;
            const T gh = P.g * hbar;
            const T rs = trsqrt(gh);
            R[0] = u; R[1] = v; R[2] = gh * rs; R[3] = (T)0.5 * rs;
            return;
#endif
        }
        R[0] = u; R[1] = v; R[2] = c; R[3] = (T)0.5 / c;
    }

    template <int IXY>
    __device__ __forceinline__ static bool rpn2(const Params &P, const T *ql, const T *qr,
                                                const T *al, const T *ar, T *W, T *s, T *am,
                                                T *ap, T *R) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T g = P.g;
        const T hl = ql[0], hr = qr[0];
        roe<IXY>(P, ql, qr, al, ar, R);
        const T ubar = R[0], vbar = R[1], cbar = R[2], half = R[3];
        T d0 = hr - hl, d1 = qr[mu] - ql[mu], d2 = qr[mv] - ql[mv];
        T a1 = ((ubar + cbar) * d0 - d1) * half;
        T a2 = -vbar * d0 + d2;
        T a3 = (-(ubar - cbar) * d0 + d1) * half;
        T *w1 = W, *w2 = W + 3, *w3 = W + 6;
        w1[0] = a1; w1[mu] = a1 * (ubar - cbar); w1[mv] = a1 * vbar;
        s[0] = ubar - cbar;
        w2[0] = (T)0; w2[mu] = (T)0; w2[mv] = a2;
        s[1] = ubar;
        w3[0] = a3; w3[mu] = a3 * (ubar + cbar); w3[mv] = a3 * vbar;
        s[2] = ubar + cbar;

        // entropy fix: amdq first, apdq = sum(s W) - amdq
        const T s0 = al[2 + mu] - al[5];  // u - c in the left cell
        if (ge0(s0) && gt0(s[0])) {
#pragma unroll
            for (int k = 0; k < 3; k++) am[k] = (T)0;
        } else {
            T h1 = hl + w1[0];
            T hu1 = ql[mu] + w1[mu];
            T s1 = (T)0, sfract;
            bool sonic1 = false;  // s0 < 0 < s1: transonic 1-rarefaction
            if (lt0(s0) && !no_right_sonic_point(h1, hu1, g)) {
                s1 = hu1 / h1 - tsqrt(g * h1);
                sonic1 = s1 > (T)0;
            }
            if (sonic1)
                sfract = s0 * (s1 - s[0]) / (s1 - s0);
            else if (lt0(s[0]))
                sfract = s[0];
            else
                sfract = (T)0;
#pragma unroll
            for (int k = 0; k < 3; k++) am[k] = sfract * w1[k];
            if (lt0(s[1])) {
#pragma unroll
                for (int k = 0; k < 3; k++) am[k] = am[k] + s[1] * w2[k];
                const T s03 = ar[2 + mu] + ar[5];  // u + c in the right cell
                T h3 = hr - w3[0];
                T hu3 = qr[mu] - w3[mu];
                T s3 = (T)0;
                bool sonic3 = false;  // s3 < 0 < s03: transonic 3-rarefaction
                if (gt0(s03) && !no_right_sonic_point(h3, -hu3, g)) {
                    s3 = hu3 / h3 + tsqrt(g * h3);
                    sonic3 = s3 < (T)0;
                }
                bool add = true;
                if (sonic3)
                    sfract = s3 * (s03 - s[2]) / (s03 - s3);
                else if (lt0(s[2]))
                    sfract = s[2];
                else
                    add = false;
                if (add) {
#pragma unroll
                    for (int k = 0; k < 3; k++) am[k] = am[k] + sfract * w3[k];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            T df = (T)0;
#pragma unroll
            for (int p = 0; p < 3; p++) df = df + s[p] * W[3 * p + k];
            ap[k] = df - am[k];
        }
        return false;
    }

    template <int IXY>
    __device__ __forceinline__ static void rpt2(const Params &P, const T *R, const T *asdq, T *bm,
                                                T *bp) {
        constexpr int mu = IXY, mv = 3 - IXY;
        T ubar = R[0], vbar = R[1], cbar = R[2], half = R[3];
        T a1 = ((vbar + cbar) * asdq[0] - asdq[mv]) * half;
        T a2 = asdq[mu] - ubar * asdq[0];
        T a3 = (-(vbar - cbar) * asdq[0] + asdq[mv]) * half;
        T wb[9], sb[3];
        wb[0] = a1; wb[mu] = a1 * ubar; wb[mv] = a1 * (vbar - cbar);
        sb[0] = vbar - cbar;
        wb[3] = (T)0; wb[3 + mu] = a2; wb[3 + mv] = (T)0;
        sb[1] = vbar;
        wb[6] = a3; wb[6 + mu] = a3 * ubar; wb[6 + mv] = a3 * (vbar + cbar);
        sb[2] = vbar + cbar;
        if (le0(sb[0]) && ge0(sb[2])) {
            // Subsonic across the edge (the usual case): the first wave
            // goes only down, the third only up, and the shear wave has
            // one component, so the sums of split_sum reduce to these
            // terms; the dropped terms are exact zeros.
            const T m1 = neg_part(sb[1]), p1 = pos_part(sb[1]);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                bm[k] = sb[0] * wb[k];
                bp[k] = sb[2] * wb[6 + k];
            }
            bm[mu] = bm[mu] + m1 * a2;
            bp[mu] = p1 * a2 + bp[mu];
        } else {
            split_sum<T, 3, 3>(sb, wb, bm, bp);
        }
    }
};

// ---------------------------------------------------------------------------
// Shallow water over bathymetry, f-wave form: q = (h, hu, hv), user aux (b).
// The flux difference plus the bathymetry source, delta = f(qr) - f(ql) +
// (0, g hbar (br - bl), 0), is split into f-waves along the eigenvectors of
// the Roe matrix (Bale, LeVeque, Mitran and Rossmanith, SIAM J. Sci. Comput.
// 24 (2002); upstream riemann rpn2_shallow_bathymetry_fwave.f90); the
// fluctuations are the f-waves of negative / positive speed, half each at
// speed zero.  A lake at rest (h + b constant, no velocity) gives delta = 0.
// Roe averages and the transverse split are those of RpShallow.
// aux = (b, sqrt h, hu / sqrt h, hv / sqrt h, hu / h, hv / h).
// ---------------------------------------------------------------------------
template <typename T>
struct RpShallowFwave {
    static constexpr int M = 3, MW = 3, NR = 4, NA = 6, NUA = 1;
    static constexpr bool TNB = false, FWAVE = true, CAPA = false;
    using Params = typename RpShallow<T>::Params;
    static Params make(const double *pd) { return RpShallow<T>::make(pd); }

    template <int IXY>
    __host__ __device__ static constexpr bool wnz(int p, int k) {
        return RpShallow<T>::template wnz<IXY>(p, k);
    }

    // aux[0] holds b on entry and keeps it; the depth terms follow
    __device__ __forceinline__ static void cell_aux_user(const Params &P, const T *q, T *aux) {
        T a6[6];
        RpShallow<T>::cell_aux(P, q, a6);
#pragma unroll
        for (int f = 0; f < 5; f++) aux[1 + f] = a6[f];
    }

    template <int IXY>
    __device__ __forceinline__ static bool rpn2(const Params &P, const T *ql, const T *qr,
                                                const T *al, const T *ar, T *Z, T *s, T *am,
                                                T *ap, T *R) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T g = P.g;
        const T hl = ql[0], hr = qr[0];
        if (!gt0(hl) || !gt0(hr)) {
#pragma unroll
            for (int f = 0; f < 9; f++) Z[f] = (T)0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                s[k] = am[k] = ap[k] = (T)0;
                R[k] = (T)0;
            }
            R[3] = (T)0;
            return true;
        }
        RpShallow<T>::template roe<IXY>(P, ql, qr, al + 1, ar + 1, R);
        const T ubar = R[0], vbar = R[1], cbar = R[2];
        const T ul = al[3 + mu], vl = al[3 + mv], ur = ar[3 + mu], vr = ar[3 + mv];
        const T hbar = (hl + hr) * (T)0.5;
        const T d0 = qr[mu] - ql[mu];
        const T d1 = (qr[mu] * ur + (T)0.5 * g * hr * hr) - (ql[mu] * ul + (T)0.5 * g * hl * hl) +
                     g * hbar * (ar[0] - al[0]);
        const T d2 = qr[mu] * vr - ql[mu] * vl;
        s[0] = ubar - cbar;
        s[1] = ubar;
        s[2] = ubar + cbar;
#ifdef GCLAW_STRICT
        const T b1 = (s[2] * d0 - d1) / (s[2] - s[0]);
        const T b3 = (d1 - s[0] * d0) / (s[2] - s[0]);
#else
        const T rd = rcp_fast(s[2] - s[0]);
        const T b1 = (s[2] * d0 - d1) * rd;
        const T b3 = (d1 - s[0] * d0) * rd;
#endif
        const T b2 = d2 - vbar * d0;
        T *z1 = Z, *z2 = Z + 3, *z3 = Z + 6;
        z1[0] = b1; z1[mu] = b1 * s[0]; z1[mv] = b1 * vbar;
        z2[0] = (T)0; z2[mu] = (T)0; z2[mv] = b2;
        z3[0] = b3; z3[mu] = b3 * s[2]; z3[mv] = b3 * vbar;
#pragma unroll
        for (int k = 0; k < 3; k++) am[k] = ap[k] = (T)0;
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const bool neg = lt0(s[p]), pos = gt0(s[p]);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const T z = Z[3 * p + k];
                if (neg) {
                    am[k] = am[k] + z;
                } else if (pos) {
                    ap[k] = ap[k] + z;
                } else {
                    am[k] = am[k] + (T)0.5 * z;
                    ap[k] = ap[k] + (T)0.5 * z;
                }
            }
        }
        return false;
    }

    template <int IXY>
    __device__ __forceinline__ static void rpt2(const Params &P, const T *R, const T *asdq, T *bm,
                                                T *bp) {
        RpShallow<T>::template rpt2<IXY>(P, R, asdq, bm, bp);
    }
};

// ---------------------------------------------------------------------------
// 2D Euler, Roe solver with 4 waves (acoustic u-c, entropy u, shear u,
// acoustic u+c) and optional Harten-Hyman entropy fix: q = (rho, rhou, rhov, E).
// Roe state kept for rpt2: R = (u, v, enth, u2v2, a, g1a2, euv).
// ---------------------------------------------------------------------------
template <typename T>
struct RpEuler {
    static constexpr int M = 4, MW = 4, NR = 7, NA = 8, NUA = 0;
    static constexpr bool TNB = false, FWAVE = false, CAPA = false;
    struct Params {
        T gamma, gamma1;
        int efix;
    };
    static Params make(const double *pd) {
        return Params{(T)pd[0], (T)(pd[0] - 1.0), pd[1] != 0.0 ? 1 : 0};
    }

    // the shear wave (third) has no density and no normal momentum
    template <int IXY>
    __host__ __device__ static constexpr bool wnz(int p, int k) {
        return p != 2 || (k != 0 && k != IXY);
    }

    __device__ __forceinline__ static T pressure(T gamma1, const T *q) {
        return gamma1 * (q[3] - qdiv((T)0.5 * (q[1] * q[1] + q[2] * q[2]), q[0]));
    }

    // aux = (sqrt rho, p, rho u / sqrt rho, rho v / sqrt rho, (E + p) / sqrt rho,
    //        u, v, c)
    __device__ __forceinline__ static void cell_aux(const Params &P, const T *q, T *aux) {
        const T rs = tsqrt(q[0]);
        const T p = pressure(P.gamma1, q);
        aux[0] = rs;
        aux[1] = p;
        aux[2] = qdiv(q[1], rs);
        aux[3] = qdiv(q[2], rs);
        aux[4] = qdiv(q[3] + p, rs);
        aux[5] = qdiv(q[1], q[0]);
        aux[6] = qdiv(q[2], q[0]);
        aux[7] = tsqrt(qdiv(P.gamma * p, q[0]));
    }

    template <int IXY>
    __device__ __forceinline__ static bool rpn2(const Params &P, const T *ql, const T *qr,
                                                const T *al, const T *ar, T *W, T *s, T *am,
                                                T *ap, T *R) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T gamma = P.gamma, gamma1 = P.gamma1;
        const T pl = al[1];
        const T pr = ar[1];
        T u, v, enth;
        if (sizeof(T) == 4 && (ql[0] < (T)1e-3 || qr[0] < (T)1e-3)) {
            // near-vacuum states: Roe averages in FP64
            double rl = sqrt((double)ql[0]), rr = sqrt((double)qr[0]), rs = rl + rr;
            u = (T)(((double)ql[mu] / rl + (double)qr[mu] / rr) / rs);
            v = (T)(((double)ql[mv] / rl + (double)qr[mv] / rr) / rs);
            enth = (T)((((double)ql[3] + (double)pl) / rl + ((double)qr[3] + (double)pr) / rr) / rs);
        } else {
            const T rhsq2 = al[0] + ar[0];
            u = qdiv(al[1 + mu] + ar[1 + mu], rhsq2);
            v = qdiv(al[1 + mv] + ar[1 + mv], rhsq2);
            enth = qdiv(al[4] + ar[4], rhsq2);
        }
        T u2v2 = u * u + v * v;
        T c2 = gamma1 * (enth - (T)0.5 * u2v2);
        bool bad = !(c2 > (T)0);
        T a = tsqrt(c2);
        T g1a2 = qdiv(gamma1, c2);
        T euv = enth - u2v2;
        R[0] = u; R[1] = v; R[2] = enth; R[3] = u2v2; R[4] = a; R[5] = g1a2; R[6] = euv;
        T d0 = qr[0] - ql[0], dmu = qr[mu] - ql[mu], dmv = qr[mv] - ql[mv], d3 = qr[3] - ql[3];
        T a3 = g1a2 * (euv * d0 + u * dmu + v * dmv - d3);
        T a2 = dmv - v * d0;
        T a4 = qdiv(dmu + (a - u) * d0 - a * a3, (T)2 * a);
        T a1 = d0 - a3 - a4;
        T *w1 = W, *w2 = W + 4, *w3 = W + 8, *w4 = W + 12;
        w1[0] = a1; w1[mu] = a1 * (u - a); w1[mv] = a1 * v; w1[3] = a1 * (enth - u * a);
        s[0] = u - a;
        w2[0] = a3; w2[mu] = a3 * u; w2[mv] = a3 * v; w2[3] = a3 * (T)0.5 * u2v2;
        s[1] = u;
        w3[0] = (T)0; w3[mu] = (T)0; w3[mv] = a2; w3[3] = a2 * v;
        s[2] = u;
        w4[0] = a4; w4[mu] = a4 * (u + a); w4[mv] = a4 * v; w4[3] = a4 * (enth + u * a);
        s[3] = u + a;

        if (!P.efix) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                am[k] = (T)0;
                ap[k] = (T)0;
            }
#pragma unroll
            for (int p = 0; p < 4; p++) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (s[p] < (T)0)
                        am[k] = am[k] + s[p] * W[4 * p + k];
                    else
                        ap[k] = ap[k] + s[p] * W[4 * p + k];
                }
            }
            return bad;
        }
        const T s0 = al[4 + mu] - al[7];  // u - c in the left cell
        if (s0 >= (T)0 && s[0] > (T)0) {
#pragma unroll
            for (int k = 0; k < 4; k++) am[k] = (T)0;
        } else {
            T rho1 = ql[0] + w1[0];
            T rhou1 = ql[mu] + w1[mu];
            T rhov1 = ql[mv] + w1[mv];
            T en1 = ql[3] + w1[3];
            T p1 = gamma1 * (en1 - qdiv((T)0.5 * (rhou1 * rhou1 + rhov1 * rhov1), rho1));
            T c1 = tsqrt(qdiv(gamma * p1, rho1));
            T s1 = qdiv(rhou1, rho1) - c1;
            T sfract;
            if (s0 < (T)0 && s1 > (T)0)
                sfract = s0 * (s1 - s[0]) / (s1 - s0);
            else if (s[0] < (T)0)
                sfract = s[0];
            else
                sfract = (T)0;
#pragma unroll
            for (int k = 0; k < 4; k++) am[k] = sfract * w1[k];
            if (s[1] < (T)0) {
#pragma unroll
                for (int k = 0; k < 4; k++) am[k] = am[k] + s[1] * w2[k];
#pragma unroll
                for (int k = 0; k < 4; k++) am[k] = am[k] + s[2] * w3[k];
                const T s3 = ar[4 + mu] + ar[7];  // u + c in the right cell
                T rho2 = qr[0] - w4[0];
                T rhou2 = qr[mu] - w4[mu];
                T rhov2 = qr[mv] - w4[mv];
                T en2 = qr[3] - w4[3];
                T p2 = gamma1 * (en2 - qdiv((T)0.5 * (rhou2 * rhou2 + rhov2 * rhov2), rho2));
                T cc2 = tsqrt(qdiv(gamma * p2, rho2));
                T s2 = qdiv(rhou2, rho2) + cc2;
                bool add = true;
                if (s2 < (T)0 && s3 > (T)0)
                    sfract = s2 * (s3 - s[3]) / (s3 - s2);
                else if (s[3] < (T)0)
                    sfract = s[3];
                else
                    add = false;
                if (add) {
#pragma unroll
                    for (int k = 0; k < 4; k++) am[k] = am[k] + sfract * w4[k];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            T df = (T)0;
#pragma unroll
            for (int p = 0; p < 4; p++) df = df + s[p] * W[4 * p + k];
            ap[k] = df - am[k];
        }
        return bad;
    }

    template <int IXY>
    __device__ __forceinline__ static void rpt2(const Params &P, const T *R, const T *asdq, T *bm,
                                                T *bp) {
        constexpr int mu = IXY, mv = 3 - IXY;
        T u = R[0], v = R[1], enth = R[2], u2v2 = R[3], a = R[4], g1a2 = R[5], euv = R[6];
        T a3 = g1a2 * (euv * asdq[0] + u * asdq[mu] + v * asdq[mv] - asdq[3]);
        T a2 = asdq[mu] - u * asdq[0];
        T a4 = qdiv(asdq[mv] + (a - v) * asdq[0] - a * a3, (T)2 * a);
        T a1 = asdq[0] - a3 - a4;
        T wb[16], sb[4];
        wb[0] = a1; wb[mu] = a1 * u; wb[mv] = a1 * (v - a); wb[3] = a1 * (enth - v * a);
        sb[0] = v - a;
        wb[4] = a3; wb[4 + mu] = a3 * u; wb[4 + mv] = a3 * v; wb[7] = a3 * (T)0.5 * u2v2;
        sb[1] = v;
        wb[8] = (T)0; wb[8 + mu] = a2; wb[8 + mv] = (T)0; wb[11] = a2 * u;
        sb[2] = v;
        wb[12] = a4; wb[12 + mu] = a4 * u; wb[12 + mv] = a4 * (v + a); wb[15] = a4 * (enth + v * a);
        sb[3] = v + a;
        if (le0(sb[0]) && ge0(sb[3])) {
            // Subsonic across the edge: the first acoustic wave goes only
            // down, the second only up; the entropy and shear waves share
            // speed v.  The terms dropped from split_sum's sums are exact
            // zeros (including the shear wave's zero density and transverse
            // momentum).
            const T m = neg_part(v), p = pos_part(v);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                T lo = sb[0] * wb[k] + m * wb[4 + k];
                T hi = p * wb[4 + k];
                if (k == mu || k == 3) {
                    lo = lo + m * wb[8 + k];
                    hi = hi + p * wb[8 + k];
                }
                bm[k] = lo;
                bp[k] = hi + sb[3] * wb[12 + k];
            }
        } else {
            split_sum<T, 4, 4>(sb, wb, bm, bp);
        }
    }
};

// Wave limiter phi(theta): 1 minmod, 2 superbee, 3 van Leer, 4 MC.
template <typename T>
__device__ __forceinline__ T philim(int id, T r) {
    switch (id) {
    case 1: return tmax((T)0, tmin((T)1, r));
    case 2: return tmax((T)0, tmax(tmin((T)1, (T)2 * r), tmin((T)2, r)));
    case 3: return (r + tabs(r)) / ((T)1 + tabs(r));
    case 4: {
        T c = ((T)1 + r) / (T)2;
        return tmax((T)0, tmin(c, tmin((T)2, (T)2 * r)));
    }
    default: return (T)1;
    }
}

// philim for theta in (0, +inf]: every operand of the min / max is then in
// [+0, +inf] and the outer max with 0 is the identity, so the same values
// come from nnmin / nnmax.
template <typename T>
__device__ __forceinline__ T philim_pos(int id, T r) {
    switch (id) {
    case 1: return nnmin((T)1, r);
    case 2: return nnmax(nnmin((T)1, (T)2 * r), nnmin((T)2, r));
    case 3: return (r + r) / ((T)1 + r);
    case 4: {
        T c = ((T)1 + r) / (T)2;
        return nnmin(c, nnmin((T)2, (T)2 * r));
    }
    default: return (T)1;
    }
}

}  // namespace gclaw
