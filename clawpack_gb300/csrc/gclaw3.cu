// gclaw3.cu -- the classic unsplit 3D wave-propagation step (PyClaw
// ClawSolver3D / classic3 step3 + flux3; Langseth and LeVeque, J. Comput.
// Phys. 165 (2000)) on GB300, FP64.
//
// One step is three sweeps (x, y, z); each sweep is three kernels over the
// whole grid, staged through a caller-provided workspace in HBM:
//   k_edges   one thread per edge: rpn3 of the two cells, storing the waves,
//             speeds and fluctuations, and the sweep's Courant numbers;
//   k_chains  one thread per edge: the limiter (against the neighbouring
//             edges' unlimited waves along the sweep), the correction flux,
//             and the transverse chains of A-dQ and A+dQ: rpt3 splits in
//             both transverse directions and, with transverse_waves 11 or
//             22, the rptt3 corner terms, stored as the values each chain
//             adds to the transverse flux entries of its cell;
//   k_update  one thread per cell: adds, in a fixed order, the first-order
//             term, the correction-flux difference and the transverse-flux
//             terms of the 3x3 slices around the cell.
// Edge records live on the box of positions [-1, n+1]^3 (x fastest, one
// field per plane), so consecutive threads touch consecutive x positions in
// every sweep.  The operations and their order are those of the CPU oracle,
// so the -fmad=false build reproduces it bit for bit.  The last block of the
// z-sweep's update applies PyClaw's evolve_to_time rules to the gclaw_ctrl
// block (finish_step), as the 2D step does.
#include <cuda_runtime.h>

#include "gclaw.h"
#include "gclaw3.h"
#include "gclaw_step_impl.cuh"

namespace gclaw {
namespace g3 {

constexpr int NT3 = 256;

struct Args3 {
    const double *qin[2];
    double *qout[2];
    double *qtmp;  // dimensionally split steps: the state between the y- and z-sweeps
    int split;     // 1: each sweep starts from the previous one's result
    gclaw_ctrl *ctrl;
    void *ws;  // edge records, in the arithmetic type of the step
    double dt, d[3];
    int n[3];
    int bc_lo[3], bc_hi[3];
    int mthlim, order, tw, ctrl_mode;
    long long npos;  // edge-box positions (n0 + 3)(n1 + 3)(n2 + 3), below 2^31
    Divisor box_x, box_y, cell_x, cell_y;  // n0 + 3, n1 + 3, n0, n1
    Divisor pen0, pen1;  // k_pencil: cells along its two pencil axes
    long long npen;      // k_pencil: threads (pencils x chunks)
};

// Box position idx -> (x, y, z), each in [-1, n + 1].
__device__ __forceinline__ void box_coords(const Args3 &a, unsigned idx, int p[3]) {
    const unsigned r = udiv(idx, a.box_x), z = udiv(r, a.box_y);
    p[0] = (int)(idx - r * (unsigned)a.box_x.d) - 1;
    p[1] = (int)(r - z * (unsigned)a.box_y.d) - 1;
    p[2] = (int)z - 1;
}

// Constant-coefficient acoustics, q = (p, u, v, w); the velocity along axis
// a is q[1 + a] (upstream riemann rpn3/rpt3/rptt3_acoustics.f90).
template <typename T>
struct Rp3Acoustics {
    static constexpr int M = 4, MW = 2, NR = 0;
    struct Params {
        T cc, zz, hz;  // hz = 1 / (2 zz)
    };
    static Params make(const double *pd) {
        return Params{(T)pd[2], (T)pd[3], (T)(1.0 / (2.0 * pd[3]))};
    }
    // The characteristic amplitude (x + zz y) / (2 zz): GCLAW_STRICT divides
    // as the reference writes it, otherwise one multiply by 1 / (2 zz).
    __device__ __forceinline__ static T amp(const Params &P, T x) {
#ifdef GCLAW_STRICT
        return x / ((T)2 * P.zz);
#else
        return x * P.hz;
#endif
    }

    // Components of a transverse chain's flux entries that can be nonzero in
    // sweep D: part 0 (G, faces normal to T1) or 1 (H, normal to T2); o = 1
    // is the face's own row (single transverse + corner terms), o = 0, 2 the
    // neighbouring rows (corner terms only).  Pressure and the transverse
    // velocities only: the normal velocity is never split transversally.
    template <int D>
    __host__ __device__ static constexpr bool chain_nz(int part, int o, int k) {
        constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
        if (k == 0) return true;
        if (o == 1) return k == 1 + T1 || k == 1 + T2;
        return k == 1 + (part == 0 ? T2 : T1);
    }

    template <int D>
    __device__ __forceinline__ static bool rpn3(const Params &P, const T *ql, const T *qr, T *W,
                                                T *s, T *am, T *ap, T *) {
        constexpr int mn = 1 + D;
        const T cc = P.cc, zz = P.zz;
        const T d0 = qr[0] - ql[0];
        const T d1 = qr[mn] - ql[mn];
        const T a1 = amp(P, -d0 + zz * d1);
        const T a2 = amp(P, d0 + zz * d1);
#pragma unroll
        for (int k = 0; k < 8; k++) W[k] = (T)0;
        W[0] = -a1 * zz; W[mn] = a1;
        s[0] = -cc;
        W[4] = a2 * zz; W[4 + mn] = a2;
        s[1] = cc;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            am[k] = s[0] * W[k];
            ap[k] = s[1] * W[4 + k];
        }
        return false;
    }

    // split asdq along axis t into the parts moving down (bm) and up (bp)
    template <int TA>
    __device__ __forceinline__ static void rpt3(const Params &P, const T *, const T *asdq, T *bm,
                                                T *bp) {
        constexpr int mt = 1 + TA;
        const T cc = P.cc, zz = P.zz;
        const T a1 = amp(P, -asdq[0] + zz * asdq[mt]);
        const T a2 = amp(P, asdq[0] + zz * asdq[mt]);
#pragma unroll
        for (int k = 0; k < 4; k++) bm[k] = bp[k] = (T)0;
        bm[0] = cc * a1 * zz; bm[mt] = -cc * a1;
        bp[0] = cc * a2 * zz; bp[mt] = cc * a2;
    }

    // split a fluctuation already split along T1 along T2 (constant
    // coefficients: the split along T2 does not depend on the state)
    template <int T1, int T2>
    __device__ __forceinline__ static void rptt3(const Params &P, const T *R, const T *b, T *cm,
                                                 T *cp) {
        rpt3<T2>(P, R, b, cm, cp);
    }
};

// 3D Euler, q = (rho, rho u, rho v, rho w, E), Roe solver with three wave
// families: acoustic (u_d - a), the entropy and both shear waves together
// (u_d), acoustic (u_d + a); no entropy fix (upstream riemann
// rpn3/rpt3/rptt3_euler.f90).  The Roe state of the edge, R = (u, v, w, H,
// a, (gamma-1)/a^2, H - |u|^2, |u|^2), is stored with the edge record and
// gives the transverse and corner splits their eigenstructure.
template <typename T>
struct Rp3Euler {
    static constexpr int M = 5, MW = 3, NR = 8;
    struct Params {
        T gamma1;
    };
    static Params make(const double *pd) { return Params{(T)(pd[0] - 1.0)}; }

    template <int D>
    __host__ __device__ static constexpr bool chain_nz(int, int, int) { return true; }

    __device__ __forceinline__ static T pressure(T gamma1, const T *q) {
        return gamma1 * (q[4] - qdiv((T)0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]), q[0]));
    }

    // Roe state; true if the averaged sound speed squared is not positive
    __device__ __forceinline__ static bool roe(const Params &P, const T *ql, const T *qr, T *R) {
        const T gamma1 = P.gamma1;
        const T rl = tsqrt(ql[0]), rr = tsqrt(qr[0]);
        const T pl = pressure(gamma1, ql), pr = pressure(gamma1, qr);
        const T rs = rl + rr;
#pragma unroll
        for (int k = 0; k < 3; k++) R[k] = qdiv(qdiv(ql[1 + k], rl) + qdiv(qr[1 + k], rr), rs);
        R[3] = qdiv(qdiv(ql[4] + pl, rl) + qdiv(qr[4] + pr, rr), rs);
        R[7] = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
        const T c2 = gamma1 * (R[3] - (T)0.5 * R[7]);
        R[4] = tsqrt(c2);
        R[5] = qdiv(gamma1, c2);
        R[6] = R[3] - R[7];
        return !gt0(c2);
    }

    // the three waves of vector dq along axis DD and their speeds
    template <int DD>
    __device__ __forceinline__ static void waves(const T *R, const T *dq, T *w, T *s) {
        constexpr int t1 = (DD + 1) % 3, t2 = (DD + 2) % 3;
        constexpr int mn = 1 + DD, m1 = 1 + t1, m2 = 1 + t2;
        const T un = R[DD], v1 = R[t1], v2 = R[t2], a = R[4], enth = R[3];
        const T a2 = R[5] * (R[6] * dq[0] + un * dq[mn] + v1 * dq[m1] + v2 * dq[m2] - dq[4]);
        const T a3 = dq[m1] - v1 * dq[0];
        const T a4 = dq[m2] - v2 * dq[0];
        const T a5 = qdiv(dq[mn] + (a - un) * dq[0] - a * a2, (T)2 * a);
        const T a1 = dq[0] - a2 - a5;
        T *w1 = w, *w2 = w + 5, *w3 = w + 10;
        w1[0] = a1; w1[mn] = a1 * (un - a); w1[m1] = a1 * v1; w1[m2] = a1 * v2;
        w1[4] = a1 * (enth - un * a);
        s[0] = un - a;
        w2[0] = a2; w2[mn] = a2 * un; w2[m1] = a2 * v1 + a3; w2[m2] = a2 * v2 + a4;
        w2[4] = a2 * (T)0.5 * R[7] + a3 * v1 + a4 * v2;
        s[1] = un;
        w3[0] = a5; w3[mn] = a5 * (un + a); w3[m1] = a5 * v1; w3[m2] = a5 * v2;
        w3[4] = a5 * (enth + un * a);
        s[2] = un + a;
    }

    template <int D>
    __device__ __forceinline__ static bool rpn3(const Params &P, const T *ql, const T *qr, T *W,
                                                T *s, T *am, T *ap, T *R) {
        const bool bad = roe(P, ql, qr, R);
        T dq[5];
#pragma unroll
        for (int k = 0; k < 5; k++) dq[k] = qr[k] - ql[k];
        waves<D>(R, dq, W, s);
#pragma unroll
        for (int k = 0; k < 5; k++) am[k] = ap[k] = (T)0;
#pragma unroll
        for (int p = 0; p < 3; p++) {
            const bool neg = lt0(s[p]);
#pragma unroll
            for (int k = 0; k < 5; k++) {
                if (neg) am[k] = am[k] + s[p] * W[5 * p + k];
                else ap[k] = ap[k] + s[p] * W[5 * p + k];
            }
        }
        return bad;
    }

    template <int TA>
    __device__ __forceinline__ static void rpt3(const Params &, const T *R, const T *asdq, T *bm,
                                                T *bp) {
        T w[15], sb[3];
        waves<TA>(R, asdq, w, sb);
#pragma unroll
        for (int k = 0; k < 5; k++) {
            T lo = (T)0, hi = (T)0;
#pragma unroll
            for (int p = 0; p < 3; p++) {
                lo = lo + neg_part(sb[p]) * w[5 * p + k];
                hi = hi + pos_part(sb[p]) * w[5 * p + k];
            }
            bm[k] = lo;
            bp[k] = hi;
        }
    }

    template <int T1, int T2>
    __device__ __forceinline__ static void rptt3(const Params &P, const T *R, const T *b, T *cm,
                                                 T *cp) {
        rpt3<T2>(P, R, b, cm, cp);
    }
};

// Slot of chain entry (part, face s, row o, component k) among the entries
// that can be nonzero in sweep D, or -1; and the number of slots.
template <class RP, int D>
__host__ __device__ constexpr int chain_slot(int part, int s, int o, int k) {
    int n = 0;
    for (int pp = 0; pp < 2; pp++)
        for (int ss = 0; ss < 2; ss++)
            for (int oo = 0; oo < 3; oo++)
                for (int kk = 0; kk < RP::M; kk++) {
                    if (!RP::template chain_nz<D>(pp, oo, kk)) continue;
                    if (pp == part && ss == s && oo == o && kk == k) return n;
                    n++;
                }
    return -1;
}
template <class RP, int D>
__host__ __device__ constexpr int chain_slots() {
    int n = 0;
    for (int pp = 0; pp < 2; pp++)
        for (int ss = 0; ss < 2; ss++)
            for (int oo = 0; oo < 3; oo++)
                for (int kk = 0; kk < RP::M; kk++) n += RP::template chain_nz<D>(pp, oo, kk);
    return n;
}

// Field planes of the workspace (doubles), per edge position: the edge
// record of k_edges, then the correction flux and the A-dQ / A+dQ chains of
// k_chains (the slots that can be nonzero; the count is the same in every
// sweep).
template <class RP>
struct Fields {
    static constexpr int M = RP::M, MW = RP::MW, NCH = chain_slots<RP, 0>();
    static_assert(NCH == chain_slots<RP, 1>() && NCH == chain_slots<RP, 2>(), "slot count");
    static constexpr int NR = RP::NR > 0 ? RP::NR : 1;
    static constexpr int W = 0, S = MW * M, AM = S + MW, AP = AM + M, R = AP + M, FA = R + NR;
    static constexpr int AMC = FA + M, APC = AMC + NCH, NF = APC + NCH;
};

// Box position of (x, y, z), each in [-1, n + 1].
__device__ __forceinline__ long long bpos(const Args3 &a, int x, int y, int z) {
    return (long long)(x + 1) +
           (long long)(a.n[0] + 3) * ((long long)(y + 1) + (long long)(a.n[1] + 3) * (z + 1));
}

// q(k) at cell (g0, g1, g2), each in [-2, n+1], through the boundary
// conditions (x, then y, then z, as the ghost fill composes them; a wall
// negates the velocity normal to it).
template <int M>
__device__ __forceinline__ double load_q3(const Args3 &a, const double *__restrict__ q, int k,
                                          int g0, int g1, int g2) {
    int g[3] = {g0, g1, g2}, si[3];
    bool neg = false;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int n = a.n[d];
        int v = min(max(g[d], -2), n + 1);
        if (v < 0) {
            const int b = a.bc_lo[d];
            if (b == GCLAW_BC_EXTRAP) v = 0;
            else if (b == GCLAW_BC_PERIODIC) v = v + n;
            else { v = -1 - v; neg = neg || (M > 1 && k == 1 + d); }
        } else if (v >= n) {
            const int b = a.bc_hi[d];
            if (b == GCLAW_BC_EXTRAP) v = n - 1;
            else if (b == GCLAW_BC_PERIODIC) v = v - n;
            else { v = 2 * n - 1 - v; neg = neg || (M > 1 && k == 1 + d); }
        }
        si[d] = v;
    }
    const double x = __ldg(q + k + (size_t)M * ((size_t)si[0] + (size_t)a.n[0] *
                                                 ((size_t)si[1] + (size_t)a.n[1] * (size_t)si[2])));
    return __longlong_as_double(__double_as_longlong(x) ^
                                (neg ? (long long)0x8000000000000000ull : 0ll));
}

// The M components of cell (g0, g1, g2) whose coordinates across axis D are
// interior and whose g[D] is in [-2, n+1], through the boundary conditions
// along D (the mapping of load_q3 for such cells, done once per cell), and
// converted to T.  Cells of an even number of components are 16-byte
// aligned and load as double2.
template <int M, int D, typename T>
__device__ __forceinline__ void load_pencil(const Args3 &a, const double *__restrict__ q, int g0,
                                            int g1, int g2, T *out) {
    int g[3] = {g0, g1, g2};
    const int n = a.n[D];
    int v = min(max(g[D], -2), n + 1);
    bool wall = false;
    if (v < 0) {
        const int b = a.bc_lo[D];
        if (b == GCLAW_BC_EXTRAP) v = 0;
        else if (b == GCLAW_BC_PERIODIC) v = v + n;
        else { v = -1 - v; wall = true; }
    } else if (v >= n) {
        const int b = a.bc_hi[D];
        if (b == GCLAW_BC_EXTRAP) v = n - 1;
        else if (b == GCLAW_BC_PERIODIC) v = v - n;
        else { v = 2 * n - 1 - v; wall = true; }
    }
    g[D] = v;
    const double *c = q + (size_t)M * ((size_t)g[0] + (size_t)a.n[0] *
                                       ((size_t)g[1] + (size_t)a.n[1] * (size_t)g[2]));
    double x[M];
    if (M % 2 == 0) {
#pragma unroll
        for (int k = 0; k < M; k += 2) {
            const double2 u = __ldg(reinterpret_cast<const double2 *>(c + k));
            x[k] = u.x;
            x[k + 1] = u.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < M; k++) x[k] = __ldg(c + k);
    }
    if (M > 1 + D && wall) x[1 + D] = __longlong_as_double(__double_as_longlong(x[1 + D]) ^
                                                          (long long)0x8000000000000000ull);
#pragma unroll
    for (int k = 0; k < M; k++) out[k] = from_double<T>(x[k]);
}

// M doubles to cell offset o (16-byte aligned when M is even)
template <int M>
__device__ __forceinline__ void store_cell(double *dst, size_t o, const double *v) {
    if (M % 2 == 0) {
#pragma unroll
        for (int k = 0; k < M; k += 2)
            *reinterpret_cast<double2 *>(dst + o + k) = make_double2(v[k], v[k + 1]);
    } else {
#pragma unroll
        for (int k = 0; k < M; k++) dst[o + k] = v[k];
    }
}
template <int M>
__device__ __forceinline__ void load_cell(const double *src, size_t o, double *v) {
    if (M % 2 == 0) {
#pragma unroll
        for (int k = 0; k < M; k += 2) {
            const double2 u = *reinterpret_cast<const double2 *>(src + o + k);
            v[k] = u.x;
            v[k + 1] = u.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < M; k++) v[k] = src[o + k];
    }
}

// The M components of cell (g0, g1, g2), each coordinate in [-2, n+1],
// through the boundary conditions of all three axes (load_q3's mapping, done
// once per cell), converted to T.
template <int M, typename T>
__device__ __forceinline__ void load_cell3(const Args3 &a, const double *__restrict__ q, int g0,
                                           int g1, int g2, T *out) {
    int g[3] = {g0, g1, g2};
    unsigned negm = 0u;  // components negated by walls
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int n = a.n[d];
        int v = min(max(g[d], -2), n + 1);
        if (v < 0) {
            const int b = a.bc_lo[d];
            if (b == GCLAW_BC_EXTRAP) v = 0;
            else if (b == GCLAW_BC_PERIODIC) v = v + n;
            else { v = -1 - v; negm |= 1u << (1 + d); }
        } else if (v >= n) {
            const int b = a.bc_hi[d];
            if (b == GCLAW_BC_EXTRAP) v = n - 1;
            else if (b == GCLAW_BC_PERIODIC) v = v - n;
            else { v = 2 * n - 1 - v; negm |= 1u << (1 + d); }
        }
        g[d] = v;
    }
    const double *c = q + (size_t)M * ((size_t)g[0] + (size_t)a.n[0] *
                                       ((size_t)g[1] + (size_t)a.n[1] * (size_t)g[2]));
#pragma unroll
    for (int k = 0; k < M; k++) {
        const double x = __ldg(c + k);
        const bool neg = M > 1 && ((negm >> k) & 1u);
        out[k] = from_double<T>(__longlong_as_double(__double_as_longlong(x) ^
                                                     (neg ? (long long)0x8000000000000000ull : 0ll)));
    }
}

// The state a sweep starts from and the one it writes.  Unsplit: every
// sweep reads the old state, the x-sweep writes the new one and the others
// add to it.  Split (x, y, z in turn): old -> new -> tmp -> new.
__device__ __forceinline__ const double *sweep_in(const Args3 &a, int d, int par) {
    if (!a.split || d == 0) return a.qin[par];
    return d == 1 ? a.qout[par] : a.qtmp;
}
__device__ __forceinline__ double *sweep_out(const Args3 &a, int d, int par) {
    return a.split && d == 1 ? a.qtmp : a.qout[par];
}

// dt, parity and skip flag of this launch (device time-step control).
struct Launch {
    double dt;
    int par, skip;
};
__device__ __forceinline__ Launch launch_state(const Args3 &a) {
    __shared__ double s_dt;
    __shared__ int s_par, s_skip;
    if (threadIdx.x == 0) {
        if (a.ctrl_mode) {
            const volatile gclaw_ctrl *c = a.ctrl;
            s_skip = c->done;
            s_dt = c->dt;
            s_par = c->parity;
        } else {
            s_skip = 0;
            s_dt = a.dt;
            s_par = 0;
        }
    }
    __syncthreads();
    return Launch{s_dt, s_par, s_skip};
}

// ---- k_edges: normal Riemann problems ---------------------------------------
template <template <typename> class RPT, int D, typename T>
__global__ void __launch_bounds__(NT3) k_edges(const Args3 a, const typename RPT<T>::Params P) {
    using RP = RPT<T>;
    using F = Fields<RP>;
    constexpr int M = RP::M, MW = RP::MW;
    constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
    const Launch L = launch_state(a);
    if (L.skip) return;
    const double *__restrict__ qin = sweep_in(a, D, L.par);
    const T dtdn = (T)(L.dt / a.d[D]);
    T cmax = (T)0;
    bool bad = false;
    const long long idx = (long long)blockIdx.x * NT3 + threadIdx.x;
    if (idx < a.npos) {
        int p[3];
        box_coords(a, (unsigned)idx, p);
        int l[3] = {p[0], p[1], p[2]};
        l[D] -= 1;
        T ql[M], qr[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            ql[k] = from_double<T>(load_q3<M>(a, qin, k, l[0], l[1], l[2]));
            qr[k] = from_double<T>(load_q3<M>(a, qin, k, p[0], p[1], p[2]));
        }
        T W[MW * M], s[MW], am[M], ap[M], R[F::NR];
        const bool eb = RP::template rpn3<D>(P, ql, qr, W, s, am, ap, R);
        T *ws = static_cast<T *>(a.ws);
        const long long np = a.npos;
#pragma unroll
        for (int f = 0; f < MW * M; f++) ws[(F::W + f) * np + idx] = W[f];
#pragma unroll
        for (int q = 0; q < MW; q++) ws[(F::S + q) * np + idx] = s[q];
#pragma unroll
        for (int k = 0; k < M; k++) {
            ws[(F::AM + k) * np + idx] = am[k];
            ws[(F::AP + k) * np + idx] = ap[k];
        }
#pragma unroll
        for (int r = 0; r < RP::NR; r++) ws[(F::R + r) * np + idx] = R[r];
        // Courant numbers of the edges 0..n along the sweep in every slice
        // (ghost slices included, as the serial sweep counts them)
        // non-physical states on any edge of the slices the sweep uses
        if (p[T1] <= a.n[T1] && p[T2] <= a.n[T2]) bad |= eb;
        if (p[D] >= 0 && p[D] <= a.n[D] && p[T1] <= a.n[T1] && p[T2] <= a.n[T2]) {
#pragma unroll
            for (int q = 0; q < MW; q++) {
                bad |= isnan_v(s[q]);
                cmax = max_abs(cmax, dtdn * s[q]);
            }
        }
    }
    // block max and flag, then one atomic each
    __shared__ T s_red[NT3 / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cmax = tmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = cmax;
    const int any = __syncthreads_or(bad ? 1 : 0);
    if (threadIdx.x == 0) {
        for (int w = 1; w < NT3 / 32; w++) cmax = tmax(cmax, s_red[w]);
        const double c = (double)cmax;
        if (c > 0.0) atomicMax(&a.ctrl->smax_bits[0], (unsigned long long)__double_as_longlong(c));
        if (any) atomicOr(&a.ctrl->flags, 1u);
    }
}

// ---- k_chains: limiter, correction flux, transverse chains -----------------
template <class RP, int D, typename T>
__device__ __forceinline__ void chain(const typename RP::Params &P, const T *R, const T *asdq,
                                      bool dbl, T h, T f1, T f2, T *ws, long long np,
                                      long long idx, int base) {
    constexpr int M = RP::M;
    constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
    T bm[M], bp[M], cm[M], cp[M];
    RP::template rpt3<T1>(P, R, asdq, bm, bp);
    RP::template rpt3<T2>(P, R, asdq, cm, cp);
    T g[2][3][M], hh[2][3][M];
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
        for (int o = 0; o < 3; o++)
#pragma unroll
            for (int k = 0; k < M; k++) g[s][o][k] = hh[s][o][k] = (T)0;
#pragma unroll
    for (int k = 0; k < M; k++) {
        g[0][1][k] = (T)0 - h * bm[k];
        g[1][1][k] = (T)0 - h * bp[k];
        hh[0][1][k] = (T)0 - h * cm[k];
        hh[1][1][k] = (T)0 - h * cp[k];
    }
    if (dbl) {
        T cmb[M], cpb[M];
#pragma unroll
        for (int s = 0; s < 2; s++) {
            RP::template rptt3<T1, T2>(P, R, s ? bp : bm, cmb, cpb);
#pragma unroll
            for (int k = 0; k < M; k++) {
                g[s][1][k] = g[s][1][k] + f2 * (cpb[k] - cmb[k]);
                g[s][2][k] = (T)0 - f2 * cpb[k];
                g[s][0][k] = (T)0 + f2 * cmb[k];
            }
        }
#pragma unroll
        for (int s = 0; s < 2; s++) {
            RP::template rptt3<T2, T1>(P, R, s ? cp : cm, cmb, cpb);
#pragma unroll
            for (int k = 0; k < M; k++) {
                hh[s][1][k] = hh[s][1][k] + f1 * (cpb[k] - cmb[k]);
                hh[s][2][k] = (T)0 - f1 * cpb[k];
                hh[s][0][k] = (T)0 + f1 * cmb[k];
            }
        }
    }
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
        for (int o = 0; o < 3; o++)
#pragma unroll
            for (int k = 0; k < M; k++) {
                if (RP::template chain_nz<D>(0, o, k))
                    ws[(long long)(base + chain_slot<RP, D>(0, s, o, k)) * np + idx] = g[s][o][k];
                if (RP::template chain_nz<D>(1, o, k))
                    ws[(long long)(base + chain_slot<RP, D>(1, s, o, k)) * np + idx] = hh[s][o][k];
            }
}

template <template <typename> class RPT, int D, typename T>
__global__ void __launch_bounds__(NT3) k_chains(const Args3 a, const typename RPT<T>::Params P) {
    using RP = RPT<T>;
    using F = Fields<RP>;
    constexpr int M = RP::M, MW = RP::MW;
    constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
    const Launch L = launch_state(a);
    if (L.skip) return;
    const long long idx = (long long)blockIdx.x * NT3 + threadIdx.x;
    if (idx >= a.npos) return;
    const int X = a.n[0] + 3, Y = a.n[1] + 3;
    int p[3];
    box_coords(a, (unsigned)idx, p);
    // edges 0..n along the sweep, slices -1..n across it
    if (p[D] < 0 || p[D] > a.n[D] || p[T1] > a.n[T1] || p[T2] > a.n[T2]) return;
    T *ws = static_cast<T *>(a.ws);
    const long long np = a.npos;
    long long stepd = 1;
    if (D >= 1) stepd *= X;
    if (D >= 2) stepd *= Y;
    const T dtdn = (T)(L.dt / a.d[D]), dtt1 = (T)(L.dt / a.d[T1]), dtt2 = (T)(L.dt / a.d[T2]);

    T W[MW * M], s[MW], cq[M];
#pragma unroll
    for (int f = 0; f < MW * M; f++) W[f] = ws[(F::W + f) * np + idx];
#pragma unroll
    for (int q = 0; q < MW; q++) s[q] = ws[(F::S + q) * np + idx];
#pragma unroll
    for (int k = 0; k < M; k++) cq[k] = (T)0;
    if (a.order == 2) {
#pragma unroll
        for (int q = 0; q < MW; q++) {
            const int lim = (a.mthlim >> (8 * q)) & 0xff;
            if (lim == 0) continue;
            T wn2 = (T)0;
#pragma unroll
            for (int k = 0; k < M; k++) wn2 = wn2 + W[q * M + k] * W[q * M + k];
            if (eq0(wn2)) continue;
            T dot = (T)0;
            if (gt0(s[q])) {  // upwind: the edge before
#pragma unroll
                for (int k = 0; k < M; k++)
                    dot = dot + ws[(F::W + q * M + k) * np + idx - stepd] * W[q * M + k];
            } else {
#pragma unroll
                for (int k = 0; k < M; k++)
                    dot = dot + W[q * M + k] * ws[(F::W + q * M + k) * np + idx + stepd];
            }
            T phi = (T)0;
            if (!le0(dot)) {
                const T th = qdiv(dot, wn2);
                phi = gt0(th) ? philim_pos<T>(lim, th) : philim<T>(lim, th);
            }
#pragma unroll
            for (int k = 0; k < M; k++) W[q * M + k] = phi * W[q * M + k];
        }
        const T dtave = (T)0.5 * (dtdn + dtdn);
#pragma unroll
        for (int k = 0; k < M; k++) {
            T c = (T)0;
#pragma unroll
            for (int q = 0; q < MW; q++) {
                const T sa = tabs(s[q]);
                c = c + sa * ((T)1 - sa * dtave) * W[q * M + k];
            }
            cq[k] = c;
        }
    }
#pragma unroll
    for (int k = 0; k < M; k++) ws[(F::FA + k) * np + idx] = (T)0 + (T)0.5 * cq[k];

    const int single = a.tw / 10;
    const bool dbl = (a.tw % 10) > 0;
    T am[M], ap[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        am[k] = ws[(F::AM + k) * np + idx];
        ap[k] = ws[(F::AP + k) * np + idx];
        if (a.order == 2 && single == 2) {
            am[k] = am[k] + cq[k];
            ap[k] = ap[k] - cq[k];
        }
    }
    if (single > 0) {
        const T h = (T)0.5 * dtdn;
        const T sixth = (T)(1.0 / 6.0);
        const T f1 = sixth * dtdn * dtt1, f2 = sixth * dtdn * dtt2;
        T R[F::NR];
#pragma unroll
        for (int r = 0; r < RP::NR; r++) R[r] = ws[(F::R + r) * np + idx];
        chain<RP, D, T>(P, R, am, dbl, h, f1, f2, ws, np, idx, F::AMC);
        chain<RP, D, T>(P, R, ap, dbl, h, f1, f2, ws, np, idx, F::APC);
    }
}

// ---- k_update: per-cell accumulation of one sweep ---------------------------
// FP64: the terms are added to the state itself, in the oracle's order.
// FP32-bulk: they are summed in FP32 from zero and the sum is added to the
// FP64 state once.
template <template <typename> class RPT, int D, typename T>
__global__ void __launch_bounds__(NT3) k_update(const Args3 a) {
    using RP = RPT<T>;
    using F = Fields<RP>;
    constexpr int M = RP::M;
    constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
    constexpr bool F64 = sizeof(T) == 8;
    const Launch L = launch_state(a);
    if (L.skip) return;
    const long long ncell = (long long)a.n[0] * a.n[1] * a.n[2];
    const long long cid = (long long)blockIdx.x * NT3 + threadIdx.x;
    if (cid < ncell) {
        int p[3];
        const unsigned r = udiv((unsigned)cid, a.cell_x), z = udiv(r, a.cell_y);
        p[0] = (int)((unsigned)cid - r * (unsigned)a.n[0]);
        p[1] = (int)(r - z * (unsigned)a.n[1]);
        p[2] = (int)z;
        // the x-sweep starts from the old state, the others add to the new
        // one (unsplit) or start from the previous sweep's result (split)
        const double *src = a.split ? sweep_in(a, D, L.par) : D == 0 ? a.qin[L.par] : a.qout[L.par];
        double *dst = sweep_out(a, D, L.par);
        const size_t o = (size_t)M * (size_t)cid;
        const T *ws = static_cast<const T *>(a.ws);
        const long long np = a.npos;
        const T dtn = (T)(L.dt / a.d[D]), dt1 = (T)(L.dt / a.d[T1]), dt2 = (T)(L.dt / a.d[T2]);
        T v[M];
#pragma unroll
        for (int k = 0; k < M; k++) v[k] = F64 ? (T)src[o + k] : (T)0;
        const int c = p[D], A = p[T1], B = p[T2];
#pragma unroll
        for (int db = -1; db <= 1; db++)
#pragma unroll
            for (int da = -1; da <= 1; da++) {
                int e0[3];
                e0[D] = c; e0[T1] = A - da; e0[T2] = B - db;
                int e1[3] = {e0[0], e0[1], e0[2]};
                e1[D] = c + 1;
                const long long i0 = bpos(a, e0[0], e0[1], e0[2]);
                const long long i1 = bpos(a, e1[0], e1[1], e1[2]);
                // flux entry (part, face s, offset o) of this slice at cell c
                // (entries that cannot be nonzero are +0, as stored by the oracle)
                auto ent = [&](int part, int s, int off, int k) -> T {
                    const int slot = chain_slot<RP, D>(part, s, off + 1, k);
                    if (slot < 0) return ((T)0 + (T)0) + (T)0;
                    const T am = ws[(long long)(F::AMC + slot) * np + i1];
                    const T ap = ws[(long long)(F::APC + slot) * np + i0];
                    return ((T)0 + am) + ap;
                };
#pragma unroll
                for (int k = 0; k < M; k++) {
                    if (da == 0 && db == 0) {
                        const T qa = ((T)0 - dtn * ws[(F::AP + k) * np + i0]) -
                                     dtn * ws[(F::AM + k) * np + i1];
                        const T fa0 = ws[(F::FA + k) * np + i0];
                        const T fa1 = ws[(F::FA + k) * np + i1];
                        v[k] = v[k] + qa - dtn * (fa1 - fa0) -
                               dt1 * (ent(0, 1, 0, k) - ent(0, 0, 0, k)) -
                               dt2 * (ent(1, 1, 0, k) - ent(1, 0, 0, k));
                    } else {
                        const T gt = da == 0 ? (T)0 - dt1 * (ent(0, 1, db, k) - ent(0, 0, db, k))
                                     : da == 1 ? dt1 * ent(0, 1, db, k)
                                               : (T)0 - dt1 * ent(0, 0, db, k);
                        const T ht = db == 0 ? (T)0 - dt2 * (ent(1, 1, da, k) - ent(1, 0, da, k))
                                     : db == 1 ? dt2 * ent(1, 1, da, k)
                                               : (T)0 - dt2 * ent(1, 0, da, k);
                        v[k] = v[k] + gt + ht;
                    }
                }
            }
#pragma unroll
        for (int k = 0; k < M; k++)
            dst[o + k] = F64 ? (double)v[k] : src[o + k] + f2d_bits((float)v[k]);
    }
    if (D == 2) {
        // last block of the step: Courant number and evolve_to_time rules
        // (the edges reduced Courant numbers themselves, so no dt/dx factor)
        __shared__ int s_last;
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            s_last = atomicAdd(&a.ctrl->blocks_done, 1u) == gridDim.x - 1;
        }
        __syncthreads();
        if (s_last && threadIdx.x == 0) {
            __threadfence();
            finish_step(a.ctrl, a.ctrl_mode, L.dt, 1.0, 1.0);
        }
    }
}

// ---- k_pencil: a whole sweep without transverse terms ----------------------
// Without transverse terms (every dimensionally split sweep, and
// transverse_waves 0) a sweep is a set of independent 1D problems along its
// axis.  Each thread marches along a chunk of pencil_len cells (16 in FP32,
// 32 in FP64) of one pencil with
// the unlimited waves of three consecutive edges in registers: it solves the
// edge two ahead of the cell, limits the edge after the cell and updates the
// cell.  The state is read once (plus a four-cell overlap per chunk) and
// written once, and no edge record goes to HBM.  The arithmetic and its
// order are those of k_edges, k_chains and k_update without transverse
// terms.  Pencils of the ghost slices across the sweep are not visited:
// with extrapolation, periodic and wall boundaries their states are interior
// states with a transverse velocity negated, whose normal Riemann problems
// have the same speeds and the same physicality, so the Courant number and
// the status flags come out the same.
// limited correction flux fa = 0 + 0.5 cq of the edge with unlimited waves
// Wc and speeds s, between the edges with waves Wl (before) and Wr (after)
template <class RP, typename T>
__device__ __forceinline__ void limit_edge(const Args3 &a, const T *Wl, const T *Wc, const T *Wr,
                                           const T *s, T dtdn, T *fa, T *cq) {
    constexpr int M = RP::M, MW = RP::MW;
    T W[MW * M];
#pragma unroll
    for (int f = 0; f < MW * M; f++) W[f] = Wc[f];
#pragma unroll
    for (int k = 0; k < M; k++) cq[k] = (T)0;
    if (a.order == 2) {
#pragma unroll
        for (int q = 0; q < MW; q++) {
            const int lim = (a.mthlim >> (8 * q)) & 0xff;
            if (lim == 0) continue;
            T wn2 = (T)0;
#pragma unroll
            for (int k = 0; k < M; k++) wn2 = wn2 + W[q * M + k] * W[q * M + k];
            if (eq0(wn2)) continue;
            T dot = (T)0;
            if (gt0(s[q])) {
#pragma unroll
                for (int k = 0; k < M; k++) dot = dot + Wl[q * M + k] * W[q * M + k];
            } else {
#pragma unroll
                for (int k = 0; k < M; k++) dot = dot + W[q * M + k] * Wr[q * M + k];
            }
            T phi = (T)0;
            if (!le0(dot)) {
                const T th = qdiv(dot, wn2);
                phi = gt0(th) ? philim_pos<T>(lim, th) : philim<T>(lim, th);
            }
#pragma unroll
            for (int k = 0; k < M; k++) W[q * M + k] = phi * W[q * M + k];
        }
        const T dtave = (T)0.5 * (dtdn + dtdn);
#pragma unroll
        for (int k = 0; k < M; k++) {
            T c = (T)0;
#pragma unroll
            for (int q = 0; q < MW; q++) {
                const T sa = tabs(s[q]);
                c = c + sa * ((T)1 - sa * dtave) * W[q * M + k];
            }
            cq[k] = c;
        }
    }
#pragma unroll
    for (int k = 0; k < M; k++) fa[k] = (T)0 + (T)0.5 * cq[k];
}

// dt / d (rounded to T) once per block: an FP64 division per thread would
// occupy the narrow FP64 pipe of GB300 out of proportion to the sweep
template <typename T>
__device__ __forceinline__ T block_dtd(double dt, double d) {
    __shared__ T s_v;
    if (threadIdx.x == 0) s_v = (T)(dt / d);
    __syncthreads();
    return s_v;
}

// blocks per SM the marching kernel is compiled for: four (64 registers)
// for FP32 acoustics, one for FP64 Euler, whose three-edge window needs the
// whole register file, two (128 registers) otherwise
template <template <typename> class RPT, typename T>
constexpr int pencil_blocks() {
    return sizeof(T) == 8 ? (RPT<T>::M > 4 ? 1 : 2) : (RPT<T>::M > 4 ? 2 : 4);
}
// cells per chunk of the marching kernel: longer chunks in FP64, where the
// overlap's extra Riemann problems cost FP64-pipe time, shorter in FP32 for
// more threads in flight
template <typename T>
__host__ __device__ constexpr int pencil_len() { return sizeof(T) == 8 ? 32 : 16; }

template <template <typename> class RPT, int D, typename T>
__global__ void __launch_bounds__(NT3, pencil_blocks<RPT, T>()) k_pencil(const Args3 a, const typename RPT<T>::Params P) {
    using RP = RPT<T>;
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR > 0 ? RP::NR : 1;
    constexpr int A0 = D == 0 ? 1 : 0, A1 = D == 2 ? 1 : 2;
    constexpr bool F64 = sizeof(T) == 8;
    const Launch L = launch_state(a);
    if (L.skip) return;
    const double *__restrict__ qin = sweep_in(a, D, L.par);
    const double *src = a.split ? sweep_in(a, D, L.par) : D == 0 ? a.qin[L.par] : a.qout[L.par];
    double *dst = sweep_out(a, D, L.par);
    const T dtdn = block_dtd<T>(L.dt, a.d[D]);
    T cmax = (T)0;
    bool bad = false;
    const long long t = (long long)blockIdx.x * NT3 + threadIdx.x;
    if (t < a.npen) {
        int p[3];
        const unsigned r = udiv((unsigned)t, a.pen0), ch = udiv(r, a.pen1);
        p[A0] = (int)((unsigned)t - r * (unsigned)a.n[A0]);
        p[A1] = (int)(r - ch * (unsigned)a.n[A1]);
        const int n = a.n[D];
        constexpr int PL = pencil_len<T>();
        const int c0 = (int)ch * PL, c1 = min(c0 + PL, n);
        T qa[M], qb[M], R[NR], am[M], ap[M];
        T Wp[MW * M], Wc[MW * M], Wn[MW * M], Wx[MW * M];
        T sc[MW], sn[MW], sx[MW];
        T apc[M], amn[M], apn[M], fa0[M], fa1[M];
        // solve the edge e between cells e - 1 (ql) and e (qr), with the
        // Courant-number and flag bookkeeping of k_edges
        auto solve = [&](int e, const T *ql, const T *qr, T *W, T *sp, T *amo, T *apo) {
            const bool eb = RP::template rpn3<D>(P, ql, qr, W, sp, amo, apo, R);
            bad |= eb;
            if (e >= 0 && e <= n) {
#pragma unroll
                for (int q = 0; q < MW; q++) {
                    bad |= isnan_v(sp[q]);
                    cmax = max_abs(cmax, dtdn * sp[q]);
                }
            }
        };
        auto load = [&](int c, T *q) {
            int g[3] = {p[0], p[1], p[2]};
            g[D] = c;
            load_pencil<M, D, T>(a, qin, g[0], g[1], g[2], q);
        };
        load(c0 - 2, qa);
        load(c0 - 1, qb);
        solve(c0 - 1, qa, qb, Wp, sx, am, ap);
        load(c0, qa);
        solve(c0, qb, qa, Wc, sc, am, apc);
        load(c0 + 1, qb);
        solve(c0 + 1, qa, qb, Wn, sn, amn, apn);
        { T cq_[RP::M]; limit_edge<RP, T>(a, Wp, Wc, Wn, sc, dtdn, fa0, cq_); }
        // qb holds the cell after the current one; the cell after that is
        // loaded an iteration ahead, so its latency overlaps the arithmetic
        T qf[M];
        load(c0 + 2, qf);
#pragma unroll 1
        for (int c = c0; c < c1; c++) {
#pragma unroll
            for (int k = 0; k < M; k++) qa[k] = qf[k];
            if (c + 1 < c1) load(c + 3, qf);
            solve(c + 2, qb, qa, Wx, sx, am, ap);
            { T cq_[RP::M]; limit_edge<RP, T>(a, Wc, Wn, Wx, sn, dtdn, fa1, cq_); }
            int g[3] = {p[0], p[1], p[2]};
            g[D] = c;
            const size_t o = (size_t)M * ((size_t)g[0] + (size_t)a.n[0] *
                                          ((size_t)g[1] + (size_t)a.n[1] * (size_t)g[2]));
            double q0[M];
            load_cell<M>(src, o, q0);
#pragma unroll
            for (int k = 0; k < M; k++) {
                const T qd = ((T)0 - dtdn * apc[k]) - dtdn * amn[k];
                T v = F64 ? (T)q0[k] : (T)0;
                v = (v + qd - dtdn * (fa1[k] - fa0[k])) + (T)0;
                q0[k] = F64 ? (double)v : q0[k] + f2d_bits((float)v);
            }
            store_cell<M>(dst, o, q0);
#pragma unroll
            for (int f = 0; f < MW * M; f++) {
                Wc[f] = Wn[f];
                Wn[f] = Wx[f];
            }
#pragma unroll
            for (int q = 0; q < MW; q++) sn[q] = sx[q];
#pragma unroll
            for (int k = 0; k < M; k++) {
                apc[k] = apn[k];
                amn[k] = am[k];
                apn[k] = ap[k];
                fa0[k] = fa1[k];
                qb[k] = qa[k];
            }
        }
    }
    // block max and flag, then one atomic each
    __shared__ T s_red[NT3 / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cmax = tmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = cmax;
    const int any = __syncthreads_or(bad ? 1 : 0);
    if (threadIdx.x == 0) {
        for (int w = 1; w < NT3 / 32; w++) cmax = tmax(cmax, s_red[w]);
        const double c = (double)cmax;
        if (c > 0.0) atomicMax(&a.ctrl->smax_bits[0], (unsigned long long)__double_as_longlong(c));
        if (any) atomicOr(&a.ctrl->flags, 1u);
    }
    if (D == 2) {
        // last block of the step: Courant number and evolve_to_time rules
        __shared__ int s_last;
        if (threadIdx.x == 0) {
            __threadfence();
            s_last = atomicAdd(&a.ctrl->blocks_done, 1u) == gridDim.x - 1;
        }
        __syncthreads();
        if (s_last && threadIdx.x == 0) {
            __threadfence();
            finish_step(a.ctrl, a.ctrl_mode, L.dt, 1.0, 1.0);
        }
    }
}

// A sweep with the pencil across the lanes of a warp instead (the x-sweep,
// whose cells are contiguous along the pencil; the y- and z-sweeps on
// request): lane l holds cell c0 - 2 + l and the edge before it, and
// neighbours come by shuffles; along x every load is coalesced, along y and
// z consecutive warps take neighbouring lines (consecutive x).  A window
// updates the PLX = 28 cells c0 .. c0 + 27, and a warp takes NWX windows in
// a row; the same arithmetic as k_pencil.
constexpr int PLX = 28, NWX = 4;

template <template <typename> class RPT, int D, typename T>
__global__ void __launch_bounds__(NT3) k_pencil_w(const Args3 a, const typename RPT<T>::Params P) {
    using RP = RPT<T>;
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR > 0 ? RP::NR : 1;
    constexpr int A0 = D == 0 ? 1 : 0, A1 = D == 2 ? 1 : 2;
    constexpr bool F64 = sizeof(T) == 8;
    constexpr unsigned FULL = 0xffffffffu;
    const Launch L = launch_state(a);
    if (L.skip) return;
    const double *__restrict__ qin = sweep_in(a, D, L.par);
    const double *src = a.split ? sweep_in(a, D, L.par) : D == 0 ? a.qin[L.par] : a.qout[L.par];
    double *dst = sweep_out(a, D, L.par);
    const T dtdn = block_dtd<T>(L.dt, a.d[D]);
    T cmax = (T)0;
    bool bad = false;
    const int lane = threadIdx.x & 31;
    const long long win = ((long long)blockIdx.x * NT3 + threadIdx.x) >> 5;
    if (win < a.npen) {  // whole warps: npen counts warps
        int p[3];
        const unsigned r = udiv((unsigned)win, a.pen0), ch = udiv(r, a.pen1);
        p[A0] = (int)((unsigned)win - r * (unsigned)a.n[A0]);
        p[A1] = (int)(r - ch * (unsigned)a.n[A1]);
        const int n = a.n[D];
        // NWX windows one after another (warp-uniform loop)
#pragma unroll 1
        for (int wi = 0; wi < NWX; wi++) {
            const int c0 = ((int)ch * NWX + wi) * PLX;
            if (c0 >= n) break;
            const int x = c0 - 2 + lane;  // this lane's cell, and edge x before it
            const bool live = x <= n + 1;
            T q[M], ql[M];
            p[D] = min(x, n + 1);
            load_pencil<M, D, T>(a, qin, p[0], p[1], p[2], q);
#pragma unroll
            for (int k = 0; k < M; k++) ql[k] = __shfl_up_sync(FULL, q[k], 1);
            T W[MW * M], sp[MW], am[M], ap[M], R[NR];
            const bool eb = RP::template rpn3<D>(P, ql, q, W, sp, am, ap, R);
            if (lane >= 1 && live) {  // edges -1 .. n + 1
                bad |= eb;
                if (x >= 0 && x <= n) {
#pragma unroll
                    for (int qq = 0; qq < MW; qq++) {
                        bad |= isnan_v(sp[qq]);
                        cmax = max_abs(cmax, dtdn * sp[qq]);
                    }
                }
            }
            // the upwind neighbour's unlimited wave of each family
            T Wl[MW * M];
#pragma unroll
            for (int qq = 0; qq < MW; qq++) {
                const int from = gt0(sp[qq]) ? lane - 1 : lane + 1;
#pragma unroll
                for (int k = 0; k < M; k++)
                    Wl[qq * M + k] = __shfl_sync(FULL, W[qq * M + k], from & 31);
            }
            T fa[M];
            { T cq_[M]; limit_edge<RP, T>(a, Wl, W, Wl, sp, dtdn, fa, cq_); }
            T amr[M], far[M];
#pragma unroll
            for (int k = 0; k < M; k++) {
                amr[k] = __shfl_down_sync(FULL, am[k], 1);
                far[k] = __shfl_down_sync(FULL, fa[k], 1);
            }
            if (lane >= 2 && lane < 2 + PLX && x < n) {
                p[D] = x;
                const size_t o = (size_t)M * ((size_t)p[0] + (size_t)a.n[0] *
                                              ((size_t)p[1] + (size_t)a.n[1] * (size_t)p[2]));
                double q0[M];
                load_cell<M>(src, o, q0);
#pragma unroll
                for (int k = 0; k < M; k++) {
                    const T qd = ((T)0 - dtdn * ap[k]) - dtdn * amr[k];
                    T v = F64 ? (T)q0[k] : (T)0;
                    v = (v + qd - dtdn * (far[k] - fa[k])) + (T)0;
                    q0[k] = F64 ? (double)v : q0[k] + f2d_bits((float)v);
                }
                store_cell<M>(dst, o, q0);
            }
        }
    }
    // block max and flag, then one atomic each
    __shared__ T s_red[NT3 / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cmax = tmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = cmax;
    const int any = __syncthreads_or(bad ? 1 : 0);
    if (threadIdx.x == 0) {
        for (int w = 1; w < NT3 / 32; w++) cmax = tmax(cmax, s_red[w]);
        const double c = (double)cmax;
        if (c > 0.0) atomicMax(&a.ctrl->smax_bits[0], (unsigned long long)__double_as_longlong(c));
        if (any) atomicOr(&a.ctrl->flags, 1u);
    }
    if (D == 2) {
        // last block of the step: Courant number and evolve_to_time rules
        __shared__ int s_last;
        if (threadIdx.x == 0) {
            __threadfence();
            s_last = atomicAdd(&a.ctrl->blocks_done, 1u) == gridDim.x - 1;
        }
        __syncthreads();
        if (s_last && threadIdx.x == 0) {
            __threadfence();
            finish_step(a.ctrl, a.ctrl_mode, L.dt, 1.0, 1.0);
        }
    }
}

// ---- k_slab: a whole FP32-bulk sweep with transverse terms -----------------
// The staged sweep (k_edges, k_chains, k_update) moves every edge record and
// both transverse chains through HBM.  k_slab does the sweep in one kernel:
// a block holds a tile of SA x SB pencils along the sweep (the interior
// (SA-2) x (SB-2) and a one-pencil halo across it, SA along the axis that is
// contiguous in memory where the sweep is not along x; SB per solver, see
// slab_sb), one thread per pencil, marching together along a chunk of SL
// cells.  Each thread keeps
// the unlimited waves of three consecutive edges in registers (as k_pencil);
// at cell c it solves edge c+2, limits edge c+1, runs the A-dQ chain of edge
// c+1 into shared memory, and after a barrier the interior threads add to
// cell c, in k_update's order, the first-order and correction terms of their
// own pencil and the chain entries of the 3 x 3 pencils around (the A-dQ
// chains of edge c+1, the A+dQ chains of edge c); after a second barrier
// every thread stores the A+dQ chain of edge c+1 for the next cell.  The
// arithmetic and its order are those of the staged kernels, so the strict
// build stays bitwise equal to the oracle.  Halo pencils repeat their
// neighbours' edges (the price of keeping the chains on chip), and pencils
// in the ghost slices across the sweep take part exactly as the staged
// kernels' box positions do.
constexpr int SA = 32, SL = 16;
// tile height: 8 (256 threads, 70 % of them on interior pencils); 16
// (82 %, one 512-thread block per SM) measured slower for acoustics_3D at
// 192^3 (4.16 against 4.41 Gcell-updates/s), and euler_3D's 60 chain slots
// per buffer would not fit
template <template <typename> class RPT>
__host__ __device__ constexpr int slab_sb() {
    return 8;
}

// blocks per SM: three for acoustics_3D (57 KB of chain buffers each; the
// kernel fits 80 registers without spilling), one for euler_3D (123 KB)
template <template <typename> class RPT>
constexpr int slab_blocks() {
    return Fields<RPT<float>>::NCH <= 32 ? 3 : 1;
}

template <template <typename> class RPT, int D>
__global__ void __launch_bounds__(SA * slab_sb<RPT>(), slab_blocks<RPT>()) k_slab(const Args3 a,
                                                               const typename RPT<float>::Params P) {
    using T = float;
    using RP = RPT<T>;
    using F = Fields<RP>;
    constexpr int SB = slab_sb<RPT>(), NTS = SA * SB;
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR > 0 ? RP::NR : 1, NCH = F::NCH;
    constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
    constexpr int TA = D == 0 ? 1 : 0;       // tile axis across threads (fastest)
    constexpr int TB = 3 - D - TA;           // the other axis across the sweep
    extern __shared__ __align__(16) unsigned char slab_smem[];
    T *SAM = reinterpret_cast<T *>(slab_smem);  // A-dQ chains of edge c+1 [slot][thread]
    T *SAP = SAM + NCH * NTS;                   // A+dQ chains of edge c [slot][thread]
    const Launch L = launch_state(a);
    if (L.skip) return;
    __shared__ T s_dt[3];
    if (threadIdx.x == 0) {
        s_dt[0] = (T)(L.dt / a.d[D]);
        s_dt[1] = (T)(L.dt / a.d[T1]);
        s_dt[2] = (T)(L.dt / a.d[T2]);
    }
    __syncthreads();
    const T dtdn = s_dt[0], dtt1 = s_dt[1], dtt2 = s_dt[2];
    const double *__restrict__ qin = a.qin[L.par];
    const double *src = D == 0 ? a.qin[L.par] : a.qout[L.par];
    double *dst = a.qout[L.par];
    const int tid = threadIdx.x, ta = tid % SA, tb = tid / SA;
    int p[3];
    p[TA] = (int)blockIdx.x * (SA - 2) - 1 + ta;
    p[TB] = (int)blockIdx.y * (SB - 2) - 1 + tb;
    const int n = a.n[D];
    const int c0 = (int)blockIdx.z * SL, c1 = min(c0 + SL, n);
    // slices -1..n across the sweep are edge positions of the staged box;
    // threads past them (the ragged end of the last tiles) run along with
    // clamped states and count nothing
    const bool slice = p[TA] <= a.n[TA] && p[TB] <= a.n[TB];
    const bool inner = ta >= 1 && ta <= SA - 2 && tb >= 1 && tb <= SB - 2 && p[TA] < a.n[TA] &&
                       p[TB] < a.n[TB];
    const int single = a.tw / 10;
    const bool dbl = (a.tw % 10) > 0;
    const T h = (T)0.5 * dtdn;
    const T sixth = (T)(1.0 / 6.0);
    const T f1 = sixth * dtdn * dtt1, f2 = sixth * dtdn * dtt2;
    T cmax = (T)0;
    bool bad = false;

    auto load = [&](int c, T *q) {
        int g[3] = {p[0], p[1], p[2]};
        g[D] = c;
        load_cell3<M, T>(a, qin, g[0], g[1], g[2], q);
    };
    auto solve = [&](int e, const T *ql, const T *qr, T *W, T *sp, T *amo, T *apo, T *R) {
        const bool eb = RP::template rpn3<D>(P, ql, qr, W, sp, amo, apo, R);
        if (slice) {
            bad |= eb;
            if (e >= 0 && e <= n) {
#pragma unroll
                for (int q = 0; q < MW; q++) {
                    bad |= isnan_v(sp[q]);
                    cmax = max_abs(cmax, dtdn * sp[q]);
                }
            }
        }
    };
    // the fluctuation a chain splits: A-+dQ, with the correction flux folded
    // in for transverse_waves 2x at second order
    auto fold = [&](const T *x, const T *cq, T sign, T *out) {
#pragma unroll
        for (int k = 0; k < M; k++)
            out[k] = (a.order == 2 && single == 2) ? (sign > (T)0 ? x[k] + cq[k] : x[k] - cq[k]) : x[k];
    };

    T qa[M], qb[M], qf[M], am[M], ap[M], Rx[NR], Rn[NR];
    T Wp[MW * M], Wc[MW * M], Wn[MW * M], Wx[MW * M];
    T sc[MW], sn[MW], sx[MW];
    T apc[M], amn[M], apn[M], fa0[M], fa1[M], cq[M], asdq[M];
    load(c0 - 2, qa);
    load(c0 - 1, qb);
    solve(c0 - 1, qa, qb, Wp, sx, am, ap, Rx);
    load(c0, qa);
    solve(c0, qb, qa, Wc, sc, am, apc, Rx);   // Rx: the state of edge c0
    load(c0 + 1, qb);
    solve(c0 + 1, qa, qb, Wn, sn, amn, apn, Rn);
    limit_edge<RP, T>(a, Wp, Wc, Wn, sc, dtdn, fa0, cq);
    // the A+dQ chain of edge c0
    fold(apc, cq, (T)-1, asdq);
    chain<RP, D, T>(P, Rx, asdq, dbl, h, f1, f2, SAP, NTS, tid, 0);
    load(c0 + 2, qf);
#pragma unroll 1
    for (int c = c0; c < c1; c++) {
#pragma unroll
        for (int k = 0; k < M; k++) qa[k] = qf[k];
        if (c + 1 < c1) load(c + 3, qf);
        solve(c + 2, qb, qa, Wx, sx, am, ap, Rx);
        limit_edge<RP, T>(a, Wc, Wn, Wx, sn, dtdn, fa1, cq);
        // the A-dQ chain of edge c+1
        fold(amn, cq, (T)1, asdq);
        chain<RP, D, T>(P, Rn, asdq, dbl, h, f1, f2, SAM, NTS, tid, 0);
        __syncthreads();
        if (inner) {
            int g[3] = {p[0], p[1], p[2]};
            g[D] = c;
            const size_t o = (size_t)M * ((size_t)g[0] + (size_t)a.n[0] *
                                          ((size_t)g[1] + (size_t)a.n[1] * (size_t)g[2]));
            T v[M];
#pragma unroll
            for (int k = 0; k < M; k++) v[k] = (T)0;
#pragma unroll
            for (int db = -1; db <= 1; db++)
#pragma unroll
                for (int da = -1; da <= 1; da++) {
                    // pencil (T1 - da, T2 - db) of the tile
                    const int nb = T1 == TA ? tid - da - SA * db : tid - db - SA * da;
                    auto ent = [&](int part, int sd, int off, int k) -> T {
                        const int slot = chain_slot<RP, D>(part, sd, off + 1, k);
                        if (slot < 0) return ((T)0 + (T)0) + (T)0;
                        return ((T)0 + SAM[slot * NTS + nb]) + SAP[slot * NTS + nb];
                    };
#pragma unroll
                    for (int k = 0; k < M; k++) {
                        if (da == 0 && db == 0) {
                            const T qd = ((T)0 - dtdn * apc[k]) - dtdn * amn[k];
                            v[k] = v[k] + qd - dtdn * (fa1[k] - fa0[k]) -
                                   dtt1 * (ent(0, 1, 0, k) - ent(0, 0, 0, k)) -
                                   dtt2 * (ent(1, 1, 0, k) - ent(1, 0, 0, k));
                        } else {
                            const T gt = da == 0 ? (T)0 - dtt1 * (ent(0, 1, db, k) - ent(0, 0, db, k))
                                         : da == 1 ? dtt1 * ent(0, 1, db, k)
                                                   : (T)0 - dtt1 * ent(0, 0, db, k);
                            const T ht = db == 0 ? (T)0 - dtt2 * (ent(1, 1, da, k) - ent(1, 0, da, k))
                                         : db == 1 ? dtt2 * ent(1, 1, da, k)
                                                   : (T)0 - dtt2 * ent(1, 0, da, k);
                            v[k] = v[k] + gt + ht;
                        }
                    }
                }
#pragma unroll
            for (int k = 0; k < M; k++) dst[o + k] = src[o + k] + f2d_bits(v[k]);
        }
        __syncthreads();
        // the A+dQ chain of edge c+1, for the next cell
        fold(apn, cq, (T)-1, asdq);
        chain<RP, D, T>(P, Rn, asdq, dbl, h, f1, f2, SAP, NTS, tid, 0);
#pragma unroll
        for (int f = 0; f < MW * M; f++) {
            Wc[f] = Wn[f];
            Wn[f] = Wx[f];
        }
#pragma unroll
        for (int q = 0; q < MW; q++) sn[q] = sx[q];
#pragma unroll
        for (int k = 0; k < M; k++) {
            apc[k] = apn[k];
            amn[k] = am[k];
            apn[k] = ap[k];
            fa0[k] = fa1[k];
            qb[k] = qa[k];
        }
#pragma unroll
        for (int r = 0; r < NR; r++) Rn[r] = Rx[r];
    }
    // block max and flag, then one atomic each; the z-sweep's last block
    // finishes the step
    __shared__ T s_red[NTS / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cmax = tmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = cmax;
    const int any = __syncthreads_or(bad ? 1 : 0);
    if (threadIdx.x == 0) {
        for (int w = 1; w < NTS / 32; w++) cmax = tmax(cmax, s_red[w]);
        const double cm = (double)cmax;
        if (cm > 0.0) atomicMax(&a.ctrl->smax_bits[0], (unsigned long long)__double_as_longlong(cm));
        if (any) atomicOr(&a.ctrl->flags, 1u);
        if (D == 2) {
            __threadfence();
            const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
            if (atomicAdd(&a.ctrl->blocks_done, 1u) == nblocks - 1) {
                __threadfence();
                finish_step(a.ctrl, a.ctrl_mode, L.dt, 1.0, 1.0);
            }
        }
    }
}

template <template <typename> class RPT>
constexpr size_t slab_smem() {
    return sizeof(float) * 2 * (size_t)Fields<RPT<float>>::NCH * SA * slab_sb<RPT>();
}

// Kernel of the sweeps without transverse terms along y and z: 0 = default
// (marching threads), 1 = marching threads, 2 = warp windows.
static int g_pencil3 = 0;
// Kernels of the sweeps with transverse terms: 0 = default (k_slab in
// FP32-bulk, the staged kernels in FP64), 1 = the staged kernels.
static int g_unsplit3 = 0;

template <template <typename> class RPT, int D, typename T>
static int sweep(const gclaw3_solver *s, const Args3 &a, cudaStream_t st) {
    const typename RPT<T>::Params P = RPT<T>::make(s->problem_data);
    const unsigned nb = (unsigned)((a.npos + NT3 - 1) / NT3);
    const long long ncell = (long long)s->mx * s->my * s->mz;
    const unsigned nc = (unsigned)((ncell + NT3 - 1) / NT3);
    if (!a.tw) {
        // one kernel per sweep: warps across x for the x-sweep, threads
        // marching along y or z (consecutive threads at consecutive x) else
        constexpr int A0 = D == 0 ? 1 : 0, A1 = D == 2 ? 1 : 2;
        Args3 b = a;
        const int nn[3] = {s->mx, s->my, s->mz};
        const int n0 = nn[A0], n1 = nn[A1], nd = nn[D];
        b.pen0 = make_divisor(n0);
        b.pen1 = make_divisor(n1);
        // windows along x; along y and z marching threads unless windows
        // are asked for (measured slower for both solvers: euler_3D 128^3
        // FP32 5.6 vs 8.6, acoustics_3D 192^3 FP32 12.3 vs 18.5
        // Gcell-updates/s)
        const bool win = D == 0 || g_pencil3 == 2;
        if (win) {
            b.npen = (long long)n0 * n1 * ((nd + PLX * NWX - 1) / (PLX * NWX));
            const unsigned np = (unsigned)((b.npen * 32 + NT3 - 1) / NT3);
            k_pencil_w<RPT, D, T><<<np, NT3, 0, st>>>(b, P);
        } else {
            constexpr int PL = pencil_len<T>();
            b.npen = (long long)n0 * n1 * ((nd + PL - 1) / PL);
            const unsigned np = (unsigned)((b.npen + NT3 - 1) / NT3);
            k_pencil<RPT, D == 0 ? 1 : D, T><<<np, NT3, 0, st>>>(b, P);
        }
        return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
    }
    if constexpr (sizeof(T) == 4) {
        if (g_unsplit3 == 0) {
            // FP32-bulk: the fused sweep (FP64 stays on the staged kernels,
            // whose chains are bound by the FP64 pipe, where the halo
            // pencils' repeated chains would cost more than the saved traffic)
            constexpr int TA = D == 0 ? 1 : 0, TB = 3 - D - TA;
            constexpr int SB = slab_sb<RPT>(), NTS = SA * SB;
            const int nn[3] = {s->mx, s->my, s->mz};
            const dim3 grid((unsigned)((nn[TA] + SA - 3) / (SA - 2)),
                            (unsigned)((nn[TB] + SB - 3) / (SB - 2)),
                            (unsigned)((nn[D] + SL - 1) / SL));
            if (grid.y > 65535u || grid.z > 65535u) return GCLAW_ERR_ARG;
            constexpr size_t sm = slab_smem<RPT>();
            auto kern = k_slab<RPT, D>;
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
                cudaSuccess)
                return GCLAW_ERR_CUDA;
            kern<<<grid, NTS, sm, st>>>(a, P);
            return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
        }
    }
    k_edges<RPT, D, T><<<nb, NT3, 0, st>>>(a, P);
    k_chains<RPT, D, T><<<nb, NT3, 0, st>>>(a, P);
    k_update<RPT, D, T><<<nc, NT3, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

template <template <typename> class RPT, typename T>
static int step_all_t(const gclaw3_solver *s, const Args3 &a, cudaStream_t st, int nsteps) {
    for (int n = 0; n < nsteps; n++) {
        int rc = sweep<RPT, 0, T>(s, a, st);
        if (!rc) rc = sweep<RPT, 1, T>(s, a, st);
        if (!rc) rc = sweep<RPT, 2, T>(s, a, st);
        if (rc) return rc;
    }
    return GCLAW_OK;
}

// FP64, or FP32 edge records and fluxes with the FP64 state (FP32-bulk).
template <template <typename> class RPT>
static int step_all(const gclaw3_solver *s, const Args3 &a, cudaStream_t st, int nsteps) {
    return s->precision == GCLAW_PREC_FP64 ? step_all_t<RPT, double>(s, a, st, nsteps)
                                           : step_all_t<RPT, float>(s, a, st, nsteps);
}

// state arrays start on 16 bytes (the pencil sweeps move cells of an even
// number of components as double2)
static bool al16(const void *p) { return ((size_t)p & 15u) == 0; }

static long long box_positions(const gclaw3_solver *s) {
    return (long long)(s->mx + 3) * (long long)(s->my + 3) * (long long)(s->mz + 3);
}

static void fill_args(const gclaw3_solver *s, Args3 &a) {
    a.d[0] = s->dx;
    a.d[1] = s->dy;
    a.d[2] = s->dz;
    a.n[0] = s->mx;
    a.n[1] = s->my;
    a.n[2] = s->mz;
    for (int d = 0; d < 3; d++) {
        a.bc_lo[d] = s->bc_lower[d];
        a.bc_hi[d] = s->bc_upper[d];
    }
    a.mthlim = 0;
    for (int p = 0; p < 4; p++) a.mthlim |= (s->mthlim[p] & 0xff) << (8 * p);
    a.order = s->order;
    a.tw = s->transverse_waves;
    a.npos = box_positions(s);
    a.box_x = make_divisor(s->mx + 3);
    a.box_y = make_divisor(s->my + 3);
    a.cell_x = make_divisor(s->mx);
    a.cell_y = make_divisor(s->my);
}

}  // namespace g3
}  // namespace gclaw

using namespace gclaw;
using namespace gclaw::g3;

extern "C" {

int gclaw3_unsplit_kernel(int which) {
    const int prev = g_unsplit3;
    if (which >= 0 && which <= 1) g_unsplit3 = which;
    return prev;
}

int gclaw3_split_kernel(int which) {
    const int prev = g_pencil3;
    if (which >= 0 && which <= 2) g_pencil3 = which;
    return prev;
}

int gclaw3_rp_shape(int rp, int *num_eqn, int *num_waves) {
    switch (rp) {
    case GCLAW3_RP_ACOUSTICS_3D: *num_eqn = 4; *num_waves = 2; return GCLAW_OK;
    case GCLAW3_RP_EULER_3D: *num_eqn = 5; *num_waves = 3; return GCLAW_OK;
    default: return GCLAW_ERR_ARG;
    }
}

int gclaw3_check(const gclaw3_solver *s) {
    int m, mw;
    if (!s || gclaw3_rp_shape(s->rp, &m, &mw)) return GCLAW_ERR_ARG;
    if (s->mx < 2 || s->my < 2 || s->mz < 2) return GCLAW_ERR_ARG;
    if (!(s->dx > 0.0) || !(s->dy > 0.0) || !(s->dz > 0.0)) return GCLAW_ERR_ARG;
    // 32-bit position arithmetic (the workspace of a larger box would not
    // fit in HBM anyway)
    if ((double)(s->mx + 3) * (s->my + 3) * (s->mz + 3) >= 2147483648.0) return GCLAW_ERR_ARG;
    for (int d = 0; d < 3; d++) {
        if (s->bc_lower[d] == GCLAW_BC_CUSTOM || s->bc_upper[d] == GCLAW_BC_CUSTOM)
            return GCLAW_ERR_UNSUPPORTED;
        if (s->bc_lower[d] < GCLAW_BC_EXTRAP || s->bc_lower[d] > GCLAW_BC_WALL ||
            s->bc_upper[d] < GCLAW_BC_EXTRAP || s->bc_upper[d] > GCLAW_BC_WALL)
            return GCLAW_ERR_ARG;
        if ((s->bc_lower[d] == GCLAW_BC_PERIODIC) != (s->bc_upper[d] == GCLAW_BC_PERIODIC))
            return GCLAW_ERR_ARG;
    }
    for (int p = 0; p < GCLAW_MAX_WAVES; p++)
        if (s->mthlim[p] < 0 || s->mthlim[p] > 4) return GCLAW_ERR_UNSUPPORTED;
    if (s->order < 1 || s->order > 2) return GCLAW_ERR_ARG;
    const int tw = s->transverse_waves;
    if (tw != 0 && tw != 10 && tw != 11 && tw != 20 && tw != 22) return GCLAW_ERR_UNSUPPORTED;
    if (s->precision != GCLAW_PREC_FP64 && s->precision != GCLAW_PREC_FP32_BULK)
        return GCLAW_ERR_UNSUPPORTED;
    if (s->rp == GCLAW3_RP_ACOUSTICS_3D &&
        (!(s->problem_data[2] > 0.0) || !(s->problem_data[3] > 0.0)))
        return GCLAW_ERR_ARG;
    if (s->rp == GCLAW3_RP_EULER_3D && !(s->problem_data[0] > 1.0)) return GCLAW_ERR_ARG;
    return GCLAW_OK;
}

size_t gclaw3_workspace_bytes(const gclaw3_solver *s) {
    if (gclaw3_check(s)) return 0;
    const size_t elem = s->precision == GCLAW_PREC_FP64 ? sizeof(double) : sizeof(float);
    const size_t nf = s->rp == GCLAW3_RP_EULER_3D ? (size_t)Fields<Rp3Euler<double>>::NF
                                                  : (size_t)Fields<Rp3Acoustics<double>>::NF;
    return elem * nf * (size_t)box_positions(s);
}

int gclaw3_step(const gclaw3_solver *s, const double *q_dev, double *qnew_dev, double dt,
                void *ws_dev, gclaw_ctrl *ctrl_dev, void *stream) {
    int rc = gclaw3_check(s);
    if (rc) return rc;
    if (!q_dev || !qnew_dev || q_dev == qnew_dev || !ws_dev || !ctrl_dev || !(dt > 0.0) ||
        !al16(q_dev) || !al16(qnew_dev))
        return GCLAW_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(ctrl_dev, 0, sizeof(gclaw_ctrl), st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    Args3 a{};
    fill_args(s, a);
    a.qin[0] = a.qin[1] = q_dev;
    a.qout[0] = a.qout[1] = qnew_dev;
    a.ctrl = ctrl_dev;
    a.ws = ws_dev;
    a.dt = dt;
    a.ctrl_mode = 0;
    return s->rp == GCLAW3_RP_EULER_3D ? step_all<Rp3Euler>(s, a, st, 1)
                                       : step_all<Rp3Acoustics>(s, a, st, 1);
}

int gclaw3_step_split(const gclaw3_solver *s, const double *q_dev, double *qnew_dev,
                      double *qtmp_dev, double dt, void *ws_dev, gclaw_ctrl *ctrl_dev,
                      void *stream) {
    int rc = gclaw3_check(s);
    if (rc) return rc;
    if (!q_dev || !qnew_dev || !qtmp_dev || !ctrl_dev || !(dt > 0.0) || q_dev == qnew_dev ||
        qtmp_dev == q_dev || qtmp_dev == qnew_dev || !al16(q_dev) || !al16(qnew_dev) ||
        !al16(qtmp_dev))
        return GCLAW_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(ctrl_dev, 0, sizeof(gclaw_ctrl), st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    Args3 a{};
    fill_args(s, a);
    a.qin[0] = a.qin[1] = q_dev;
    a.qout[0] = a.qout[1] = qnew_dev;
    a.qtmp = qtmp_dev;
    a.split = 1;
    a.tw = 0;  // split sweeps carry no transverse terms
    a.ctrl = ctrl_dev;
    a.ws = ws_dev;
    a.dt = dt;
    a.ctrl_mode = 0;
    return s->rp == GCLAW3_RP_EULER_3D ? step_all<Rp3Euler>(s, a, st, 1)
                                       : step_all<Rp3Acoustics>(s, a, st, 1);
}

int gclaw3_advance_split(const gclaw3_solver *s, double *q0_dev, double *q1_dev,
                         double *qtmp_dev, void *ws_dev, gclaw_ctrl *ctrl_dev, int nsteps,
                         void *stream) {
    int rc = gclaw3_check(s);
    if (rc) return rc;
    if (!q0_dev || !q1_dev || !qtmp_dev || !ctrl_dev || nsteps < 0 || q0_dev == q1_dev ||
        qtmp_dev == q0_dev || qtmp_dev == q1_dev || !al16(q0_dev) || !al16(q1_dev) ||
        !al16(qtmp_dev))
        return GCLAW_ERR_ARG;
    Args3 a{};
    fill_args(s, a);
    a.qin[0] = q0_dev;
    a.qin[1] = q1_dev;
    a.qout[0] = q1_dev;
    a.qout[1] = q0_dev;
    a.qtmp = qtmp_dev;
    a.split = 1;
    a.tw = 0;
    a.ctrl = ctrl_dev;
    a.ws = ws_dev;
    a.dt = 0.0;
    a.ctrl_mode = 1;
    cudaStream_t st = (cudaStream_t)stream;
    return s->rp == GCLAW3_RP_EULER_3D ? step_all<Rp3Euler>(s, a, st, nsteps)
                                       : step_all<Rp3Acoustics>(s, a, st, nsteps);
}

int gclaw3_advance(const gclaw3_solver *s, double *q0_dev, double *q1_dev, void *ws_dev,
                   gclaw_ctrl *ctrl_dev, int nsteps, void *stream) {
    int rc = gclaw3_check(s);
    if (rc) return rc;
    if (!q0_dev || !q1_dev || q0_dev == q1_dev || !ws_dev || !ctrl_dev || nsteps < 0 ||
        !al16(q0_dev) || !al16(q1_dev))
        return GCLAW_ERR_ARG;
    Args3 a{};
    fill_args(s, a);
    a.qin[0] = q0_dev;
    a.qin[1] = q1_dev;
    a.qout[0] = q1_dev;
    a.qout[1] = q0_dev;
    a.ctrl = ctrl_dev;
    a.ws = ws_dev;
    a.dt = 0.0;
    a.ctrl_mode = 1;
    cudaStream_t st = (cudaStream_t)stream;
    return s->rp == GCLAW3_RP_EULER_3D ? step_all<Rp3Euler>(s, a, st, nsteps)
                                       : step_all<Rp3Acoustics>(s, a, st, nsteps);
}

}  // extern "C"
