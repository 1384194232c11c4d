// gclaw_adjoint.cuh -- reverse-mode (adjoint) versions of the per-edge
// pieces of the classic 2D step, written by hand.
//
// For each forward piece f: x -> y the function here takes x (recomputing
// what it needs of the forward) and the adjoint ybar and adds x^T-products
// into xbar.  Branches (limiter regime, upwind side, entropy-fix case,
// min/max of the transverse speeds) are decided exactly as the forward
// decides them on the same inputs, so the adjoint is that of the scheme
// actually run.  Supported solvers: acoustics_2D and
// shallow_roe_with_efix_2D.
//
// Notation follows gclaw_riemann.cuh: ql / qr left and right cells, W[MW][M]
// waves, s[MW] speeds, R the edge's Roe state, al / ar per-cell aux values.
#pragma once

#include "gclaw_riemann.cuh"

namespace gclaw {

// d phi / d theta of the wave limiters (same regimes as philim).
template <typename T>
__device__ __forceinline__ T philim_deriv(int id, T r) {
    switch (id) {
    case 1: return (r > (T)0 && r < (T)1) ? (T)1 : (T)0;
    case 2: {
        const T a = tmin((T)1, (T)2 * r), b = tmin((T)2, r);
        if (a >= b) return (a > (T)0 && (T)2 * r < (T)1) ? (T)2 : (T)0;
        return (b > (T)0 && r < (T)2) ? (T)1 : (T)0;
    }
    case 3:
        if (r <= (T)0) return (T)0;
        return (T)2 / (((T)1 + r) * ((T)1 + r));
    case 4: {
        const T c = ((T)1 + r) / (T)2;
        const T m = tmin(c, tmin((T)2, (T)2 * r));
        if (m <= (T)0) return (T)0;
        if (m == c) return (T)0.5;
        if (m == (T)2 * r) return (T)2;
        return (T)0;
    }
    default: return (T)0;
    }
}

// ---------------------------------------------------------------------------
// acoustics: everything is linear with constant coefficients.
// ---------------------------------------------------------------------------
template <typename T>
struct AdjAcoustics {
    using RP = RpAcoustics<T>;
    static constexpr int M = 3, MW = 2, NR = 1, NA = 1;

    __device__ __forceinline__ static void cell_aux_adj(const typename RP::Params &P,
                                                        const T *q, const T *aux, const T *auxb,
                                                        T *qb) {}

    // adjoint of rpn2 given adjoints of W, s, amdq, apdq, R
    template <int IXY>
    __device__ __forceinline__ static void rpn2_adj(const typename RP::Params &P, const T *ql,
                                                    const T *qr, const T *al, const T *ar,
                                                    const T *Wb, const T *sb, const T *amb,
                                                    const T *apb, const T *Rb, T *qlb, T *qrb,
                                                    T *alb, T *arb) {
        constexpr int mu = IXY;
        const T zz = P.zz, cc = P.cc;
        // amdq = s0 W0, apdq = s1 W1 (speeds constant)
        T a1b = (T)0, a2b = (T)0;
        // W0 = (-a1 zz, a1 @mu, 0); W1 = (a2 zz, a2 @mu, 0)
        T W0b[3], W1b[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            W0b[k] = Wb[k] + (-cc) * amb[k];
            W1b[k] = Wb[3 + k] + cc * apb[k];
        }
        a1b = -zz * W0b[0] + W0b[mu];
        a2b = zz * W1b[0] + W1b[mu];
        // a1 = (-d0 + zz d1) / (2 zz); a2 = (d0 + zz d1) / (2 zz)
        const T inv = (T)1 / ((T)2 * zz);
        const T d0b = (-a1b + a2b) * inv;
        const T d1b = (a1b + a2b) * zz * inv;
        qrb[0] += d0b;
        qlb[0] -= d0b;
        qrb[mu] += d1b;
        qlb[mu] -= d1b;
    }

    template <int IXY>
    __device__ __forceinline__ static void rpt2_adj(const typename RP::Params &P, const T *R,
                                                    const T *asdq, const T *bmb, const T *bpb,
                                                    T *asdqb, T *Rb) {
        constexpr int mv = 3 - IXY;
        const T zz = P.zz, cc = P.cc;
        // bm = (cc a1 zz, 0, -cc a1); bp = (cc a2 zz, 0, cc a2)
        const T a1b = cc * zz * bmb[0] - cc * bmb[mv];
        const T a2b = cc * zz * bpb[0] + cc * bpb[mv];
        const T inv = (T)1 / ((T)2 * zz);
        // a1 = (-as0 + zz as_mv) / (2 zz); a2 = (as0 + zz as_mv) / (2 zz)
        asdqb[0] += (-a1b + a2b) * inv;
        asdqb[mv] += (a1b + a2b) * zz * inv;
    }
};

// ---------------------------------------------------------------------------
// shallow water, Roe + Harten-Hyman entropy fix.
// aux = (sqrt h, hu/sqrt h, hv/sqrt h, hu/h, hv/h, sqrt(g h)); R = (u, v, c, 0.5/c)
// ---------------------------------------------------------------------------
template <typename T>
struct AdjShallow {
    using RP = RpShallow<T>;
    static constexpr int M = 3, MW = 3, NR = 4, NA = 6;

    // q adjoint from aux adjoints of one cell
    __device__ __forceinline__ static void cell_aux_adj(const typename RP::Params &P,
                                                        const T *q, const T *aux, const T *auxb,
                                                        T *qb) {
        // one reciprocal of sqrt(h), of h and of sqrt(g h) instead of a
        // quotient per term (the derivative of each aux value is linear in
        // these)
        const T h = q[0], hs = aux[0];
        const T ihs = (T)1 / hs, ih = (T)1 / h, ic = (T)1 / aux[5];
        // hu/hs, hv/hs
        T hsb = auxb[0];
        qb[1] += auxb[1] * ihs;
        hsb -= auxb[1] * aux[1] * ihs;
        qb[2] += auxb[2] * ihs;
        hsb -= auxb[2] * aux[2] * ihs;
        // hu/h, hv/h
        qb[1] += auxb[3] * ih;
        qb[2] += auxb[4] * ih;
        T hb = -(auxb[3] * aux[3] + auxb[4] * aux[4]) * ih;
        // sqrt(g h)
        hb += auxb[5] * P.g * (T)0.5 * ic;
        // sqrt(h)
        hb += hsb * (T)0.5 * ihs;
        qb[0] += hb;
    }

    template <int IXY>
    __device__ __forceinline__ static void rpn2_adj(const typename RP::Params &P, const T *ql,
                                                    const T *qr, const T *al, const T *ar,
                                                    const T *Wb_in, const T *sb_in,
                                                    const T *amb, const T *apb, const T *Rb_in,
                                                    T *qlb, T *qrb, T *alb, T *arb) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T g = P.g;
        // ---- forward recompute (same expressions as RpShallow::rpn2) ----
        T W[9], s[3], am[3], ap[3], R[4];
        RP::template rpn2<IXY>(P, ql, qr, al, ar, W, s, am, ap, R);
        const T u = R[0], v = R[1], c = R[2], half = R[3];
        const T hl = ql[0], hr = qr[0];
        const T d0 = hr - hl, d1 = qr[mu] - ql[mu];
        const T a1 = W[0], a2 = W[3 + mv], a3 = W[6];
        const T s0 = al[2 + mu] - al[5];
        const bool allright = (s0 >= (T)0 && s[0] > (T)0);
        T h1 = (T)0, hu1 = (T)0, s1 = (T)0, sf1 = (T)0, g1sq = (T)1;
        bool trans1 = false, go2 = false, add3 = false, trans3 = false;
        T h3 = (T)0, hu3 = (T)0, s3 = (T)0, s03 = (T)0, sf3 = (T)0, g3sq = (T)1;
        if (!allright) {
            h1 = hl + W[0];
            hu1 = ql[mu] + W[mu];
            // the intermediate speeds only where the forward's exact pre-test
            // leaves the transonic case open (the same branch decisions)
            if (lt0(s0) && !no_right_sonic_point(h1, hu1, g)) {
                g1sq = tsqrt(g * h1);
                s1 = hu1 / h1 - g1sq;
                trans1 = s1 > (T)0;
            }
            sf1 = trans1 ? s0 * (s1 - s[0]) / (s1 - s0) : (s[0] < (T)0 ? s[0] : (T)0);
            go2 = s[1] < (T)0;
            if (go2) {
                s03 = ar[2 + mu] + ar[5];
                h3 = hr - W[6];
                hu3 = qr[mu] - W[6 + mu];
                if (gt0(s03) && !no_right_sonic_point(h3, -hu3, g)) {
                    g3sq = tsqrt(g * h3);
                    s3 = hu3 / h3 + g3sq;
                    trans3 = s3 < (T)0;
                }
                add3 = trans3 || s[2] < (T)0;
                sf3 = trans3 ? s3 * (s03 - s[2]) / (s03 - s3) : s[2];
            }
        }
        // ---- reverse ----
        T Wb[9], sb[3], Rb[4];
#pragma unroll
        for (int f = 0; f < 9; f++) Wb[f] = Wb_in[f];
#pragma unroll
        for (int p = 0; p < 3; p++) sb[p] = sb_in[p];
#pragma unroll
        for (int r = 0; r < 4; r++) Rb[r] = Rb_in[r];
        // apdq = sum s W - amdq
        T amb_t[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
#pragma unroll
            for (int p = 0; p < 3; p++) {
                sb[p] += apb[k] * W[3 * p + k];
                Wb[3 * p + k] += apb[k] * s[p];
            }
            amb_t[k] = amb[k] - apb[k];
        }
        // entropy-fixed amdq
        if (!allright) {
            T sf1b = (T)0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                Wb[k] += sf1 * amb_t[k];
                sf1b += W[k] * amb_t[k];
            }
            T s0b = (T)0;
            if (go2) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    sb[1] += W[3 + k] * amb_t[k];
                    Wb[3 + k] += s[1] * amb_t[k];
                }
                if (add3) {
                    T sf3b = (T)0;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        Wb[6 + k] += sf3 * amb_t[k];
                        sf3b += W[6 + k] * amb_t[k];
                    }
                    if (trans3) {
                        const T D = s03 - s3, N = s3 * (s03 - s[2]);
                        const T s3b = sf3b * ((s03 - s[2]) / D + N / (D * D));
                        const T s03b = sf3b * (s3 / D - N / (D * D));
                        sb[2] -= sf3b * s3 / D;
                        // s03 = u + c of the right cell
                        arb[2 + mu] += s03b;
                        arb[5] += s03b;
                        // s3 = hu3 / h3 + sqrt(g h3), h3 = hr - W3_h, hu3 = qr_mu - W3_mu
                        const T dh3 = -hu3 / (h3 * h3) + g / ((T)2 * g3sq);
                        const T h3b = s3b * dh3, hu3b = s3b / h3;
                        qrb[0] += h3b;
                        Wb[6] -= h3b;
                        qrb[mu] += hu3b;
                        Wb[6 + mu] -= hu3b;
                    } else {
                        sb[2] += sf3b;
                    }
                }
            }
            if (trans1) {
                const T D = s1 - s0, N = s0 * (s1 - s[0]);
                s0b += sf1b * ((s1 - s[0]) / D + N / (D * D));
                const T s1b = sf1b * (s0 / D - N / (D * D));
                sb[0] -= sf1b * s0 / D;
                // s1 = hu1 / h1 - sqrt(g h1), h1 = hl + W1_h, hu1 = ql_mu + W1_mu
                const T dh1 = -hu1 / (h1 * h1) - g / ((T)2 * g1sq);
                const T h1b = s1b * dh1, hu1b = s1b / h1;
                qlb[0] += h1b;
                Wb[0] += h1b;
                qlb[mu] += hu1b;
                Wb[mu] += hu1b;
            } else if (s[0] < (T)0) {
                sb[0] += sf1b;
            }
            // s0 = u - c of the left cell
            alb[2 + mu] += s0b;
            alb[5] -= s0b;
        }
        // speeds s = (u - c, u, u + c)
        T ub = Rb[0] + sb[0] + sb[1] + sb[2];
        T vb = Rb[1];
        T cb = Rb[2] - sb[0] + sb[2];
        T halfb = Rb[3];
        // waves W1 = (a1, a1 (u - c), a1 v), W2 = (0, 0, a2), W3 = (a3, a3 (u + c), a3 v)
        const T a1b = Wb[0] + Wb[mu] * (u - c) + Wb[mv] * v;
        ub += a1 * Wb[mu];
        cb -= a1 * Wb[mu];
        vb += a1 * Wb[mv];
        const T a2b = Wb[3 + mv];
        const T a3b = Wb[6] + Wb[6 + mu] * (u + c) + Wb[6 + mv] * v;
        ub += a3 * Wb[6 + mu];
        cb += a3 * Wb[6 + mu];
        vb += a3 * Wb[6 + mv];
        // a1 = ((u + c) d0 - d1) half; a2 = -v d0 + d2; a3 = (-(u - c) d0 + d1) half
        T d0b = (T)0, d1b = (T)0, d2b = (T)0;
        {
            const T X1 = (u + c) * d0 - d1, X1b = a1b * half;
            halfb += a1b * X1;
            ub += X1b * d0;
            cb += X1b * d0;
            d0b += X1b * (u + c);
            d1b -= X1b;
        }
        vb -= a2b * d0;
        d0b -= a2b * v;
        d2b += a2b;
        {
            const T X3 = -(u - c) * d0 + d1, X3b = a3b * half;
            halfb += a3b * X3;
            ub -= X3b * d0;
            cb += X3b * d0;
            d0b -= X3b * (u - c);
            d1b += X3b;
        }
        qrb[0] += d0b;
        qlb[0] -= d0b;
        qrb[mu] += d1b;
        qlb[mu] -= d1b;
        qrb[mv] += d2b;
        qlb[mv] -= d2b;
        // Roe state: half = 0.5 / c; c = sqrt(g hbar); hbar = (hl + hr) / 2;
        // u = (us_l + us_r) / S, v = (vs_l + vs_r) / S, S = hs_l + hs_r
        // 1 / c = 2 half; one reciprocal of S
        cb -= halfb * half * ((T)2 * half);
        const T hbarb = cb * g * half;
        qlb[0] += (T)0.5 * hbarb;
        qrb[0] += (T)0.5 * hbarb;
        const T S = al[0] + ar[0];
        const T iS = (T)1 / S;
        const T Sb = -(ub * u + vb * v) * iS;
        const T ubS = ub * iS, vbS = vb * iS;
        alb[mu] += ubS;
        arb[mu] += ubS;
        alb[mv] += vbS;
        arb[mv] += vbS;
        alb[0] += Sb;
        arb[0] += Sb;
    }

    template <int IXY>
    __device__ __forceinline__ static void rpt2_adj(const typename RP::Params &P, const T *R,
                                                    const T *asdq, const T *bmb, const T *bpb,
                                                    T *asdqb, T *Rb) {
        constexpr int mu = IXY, mv = 3 - IXY;
        const T u = R[0], v = R[1], c = R[2], half = R[3];
        // forward recompute
        const T Y1 = (v + c) * asdq[0] - asdq[mv];
        const T a1 = Y1 * half;
        const T a2 = asdq[mu] - u * asdq[0];
        const T Y3 = -(v - c) * asdq[0] + asdq[mv];
        const T a3 = Y3 * half;
        T wb[9];
        wb[0] = a1; wb[mu] = a1 * u; wb[mv] = a1 * (v - c);
        wb[3] = (T)0; wb[3 + mu] = a2; wb[3 + mv] = (T)0;
        wb[6] = a3; wb[6 + mu] = a3 * u; wb[6 + mv] = a3 * (v + c);
        const T sbv[3] = {v - c, v, v + c};
        // bm = sum min(sb,0) wb, bp = sum max(sb,0) wb
        T wbb[9], sbb[3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const T lo = tmin(sbv[p], (T)0), hi = tmax(sbv[p], (T)0);
            T dl = (T)0, dh = (T)0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                wbb[3 * p + k] = lo * bmb[k] + hi * bpb[k];
                dl += wb[3 * p + k] * bmb[k];
                dh += wb[3 * p + k] * bpb[k];
            }
            sbb[p] = (sbv[p] < (T)0 ? dl : (T)0) + (sbv[p] > (T)0 ? dh : (T)0);
        }
        T ub = (T)0, vb = sbb[0] + sbb[1] + sbb[2], cb = -sbb[0] + sbb[2], halfb = (T)0;
        const T a1b = wbb[0] + wbb[mu] * u + wbb[mv] * (v - c);
        ub += a1 * wbb[mu];
        vb += a1 * wbb[mv];
        cb -= a1 * wbb[mv];
        const T a2b = wbb[3 + mu];
        const T a3b = wbb[6] + wbb[6 + mu] * u + wbb[6 + mv] * (v + c);
        ub += a3 * wbb[6 + mu];
        vb += a3 * wbb[6 + mv];
        cb += a3 * wbb[6 + mv];
        {
            const T Y1b = a1b * half;
            halfb += a1b * Y1;
            vb += Y1b * asdq[0];
            cb += Y1b * asdq[0];
            asdqb[0] += Y1b * (v + c);
            asdqb[mv] -= Y1b;
        }
        asdqb[mu] += a2b;
        ub -= a2b * asdq[0];
        asdqb[0] -= a2b * u;
        {
            const T Y3b = a3b * half;
            halfb += a3b * Y3;
            vb -= Y3b * asdq[0];
            cb += Y3b * asdq[0];
            asdqb[0] -= Y3b * (v - c);
            asdqb[mv] += Y3b;
        }
        Rb[0] += ub;
        Rb[1] += vb;
        Rb[2] += cb;
        Rb[3] += halfb;
    }
};

template <template <typename> class RPT>
struct AdjOf;
template <>
struct AdjOf<RpAcoustics> {
    template <typename T>
    using type = AdjAcoustics<T>;
};
template <>
struct AdjOf<RpShallow> {
    template <typename T>
    using type = AdjShallow<T>;
};

}  // namespace gclaw
