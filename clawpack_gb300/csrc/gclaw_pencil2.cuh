// gclaw_pencil2.cuh -- sweeps of the dimensionally split 2D step as 1D
// problems (PyClaw ClawSolver2D with dimensional_split = True, classic2
// step2ds: an x-sweep, the boundary conditions again, a y-sweep, no
// transverse terms).
//
// A split sweep is a set of independent 1D problems along its axis, so one
// kernel does the whole sweep with the state read once and written once and
// no edge record in shared memory or HBM:
//   p2_sweep_w  a window of 32 cells along the sweep across the lanes of a
//               warp, lane l at cell c0 - 2 + l with the edge on its left;
//               neighbours come by shuffles; a window updates 28 cells, a
//               warp takes P2_NWX windows in a row.  The x-sweep (cells
//               contiguous, every load coalesced), and the y-sweep of
//               euler_4wave_2D;
//   p2_sweep_y  (y) each thread marches along a chunk of one column,
//               consecutive threads at consecutive x, with the unlimited
//               waves of three consecutive edges in registers: it solves the
//               edge two ahead of the cell, limits the edge after it and
//               updates the cell.  The y-sweep of the three-component
//               solvers, whose windowed y-loads would touch twice the
//               cache sectors.
// The arithmetic and its order are those of step_kernel's phases with
// transverse_waves 0 (phase_rpn2, phase_limit, phase_accum), so the
// -fmad=false build stays bitwise equal to the oracle.  Columns and rows of
// the ghost slices across the sweep are not visited: with extrapolation,
// periodic and wall boundaries their states are interior states with the
// transverse velocity negated, whose normal Riemann problems have the same
// speeds and the same physicality, so max |s| and the status flags come out
// the same.  Solvers with user aux or a capacity do not take this path.
#pragma once

#include "gclaw_step_impl.cuh"

namespace gclaw {
namespace p2 {

constexpr int NTP = 256;
constexpr int P2_WIN = 28, P2_NWX = 4;

// blocks per SM the marching kernel is compiled for (registers: 65536 /
// (256 x blocks)): acoustics 4 in FP32 and 2 in FP64; shallow water 3 in
// FP32 (a few bytes of spill buy a third block); Euler 2 in FP32; the
// solvers with per-cell aux 1 in FP64
template <template <typename> class RPT, typename T>
constexpr int ycol_blocks() {
    using RP = RPT<T>;
    return sizeof(T) == 8 ? (RP::NA > 0 ? 1 : 2) : (RP::NA == 0 ? 4 : RP::M == 3 ? 3 : 2);
}
// cells per chunk of a column
template <typename T>
__host__ __device__ constexpr int ycol_len() {
    return sizeof(T) == 8 ? 32 : 16;
}

// dt, dt/dn (rounded to T), parity and skip flag of this launch
template <typename T>
struct Launch2 {
    double dt;
    T dtdn;
    int par, skip;
};
template <typename T>
__device__ __forceinline__ Launch2<T> launch2(const StepArgs &a, double dn) {
    __shared__ double s_dt;
    __shared__ T s_dtdn;
    __shared__ int s_par, s_skip;
    if (threadIdx.x == 0) {
        double dt;
        if (a.ctrl_mode) {
            const volatile gclaw_ctrl *c = a.ctrl;
            s_skip = c->done;
            dt = c->dt;
            s_par = c->parity;
        } else {
            s_skip = 0;
            dt = a.dt;
            s_par = 0;
        }
        s_dt = dt;
        s_dtdn = (T)(dt / dn);
    }
    __syncthreads();
    return Launch2<T>{s_dt, s_dtdn, s_par, s_skip};
}

// The M components of cell (i, j), the coordinate across the sweep
// interior and the one along it in [-2, n+1], through the boundary
// conditions along the sweep (load_q's mapping), converted to T.
template <int M, int IXY, typename T>
__device__ __forceinline__ void load_cell2(const StepArgs &a, const double *__restrict__ q, int i,
                                           int j, T *out) {
    const int n = IXY == 1 ? a.mx : a.my;
    int v = min(max(IXY == 1 ? i : j, -2), n + 1);
    bool wall = false;
    if (v < 0) {
        const int b = a.bc_lo[IXY - 1];
        if (b == GCLAW_BC_EXTRAP) v = 0;
        else if (b == GCLAW_BC_PERIODIC) v = v + n;
        else { v = -1 - v; wall = true; }
    } else if (v >= n) {
        const int b = a.bc_hi[IXY - 1];
        if (b == GCLAW_BC_EXTRAP) v = n - 1;
        else if (b == GCLAW_BC_PERIODIC) v = v - n;
        else { v = 2 * n - 1 - v; wall = true; }
    }
    if (IXY == 1) i = v;
    else j = v;
    const double *c = q + (size_t)M * ((size_t)i + (size_t)a.mx * (size_t)j);
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
    if (wall) x[IXY] = __longlong_as_double(__double_as_longlong(x[IXY]) ^
                                            (long long)0x8000000000000000ull);
#pragma unroll
    for (int k = 0; k < M; k++) out[k] = from_double<T>(x[k]);
}

template <int M>
__device__ __forceinline__ void load_row(const double *src, size_t o, double *v) {
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
template <int M>
__device__ __forceinline__ void store_row(double *dst, size_t o, const double *v) {
    if (M % 2 == 0) {
#pragma unroll
        for (int k = 0; k < M; k += 2)
            *reinterpret_cast<double2 *>(dst + o + k) = make_double2(v[k], v[k + 1]);
    } else {
#pragma unroll
        for (int k = 0; k < M; k++) dst[o + k] = v[k];
    }
}

// Normal Riemann problem of one edge with phase_rpn2's bookkeeping:
// non-physical states on every edge solved, NaN speeds and max |s| on
// edges 0..n; components that are zero by the eigenstructure set to +0, as
// phase_limit reads them.
template <class RP, int IXY, typename T>
__device__ __forceinline__ void solve2(const typename RP::Params &P, int e, int n, const T *ql,
                                       const T *al, const T *qr, const T *ar, T *W, T *s, T *am,
                                       T *ap, T &smax, bool &bad) {
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR > 0 ? RP::NR : 1;
    T R[NR];
    bad |= RP::template rpn2<IXY>(P, ql, qr, al, ar, W, s, am, ap, R);
#pragma unroll
    for (int f = 0; f < MW * M; f++)
        if (!RP::template wnz<IXY>(f / M, f % M)) W[f] = (T)0;
    if (e >= 0 && e <= n) {
#pragma unroll
        for (int p = 0; p < MW; p++) {
            bad |= isnan_v(s[p]);
            smax = max_abs(smax, s[p]);
        }
    }
}

// phase_limit without transverse terms: fa = 0 + 0.5 cq of the edge with
// unlimited waves Wc and speeds s, between the edges with waves Wl (before)
// and Wr (after)
template <class RP, int IXY, typename T>
__device__ __forceinline__ void limit2(int mthlim, int order, const T *Wl, const T *Wc,
                                       const T *Wr, const T *s, T dtdn, T *fa) {
    constexpr int M = RP::M, MW = RP::MW;
    T W[MW * M], cq[M];
#pragma unroll
    for (int f = 0; f < MW * M; f++) W[f] = Wc[f];
#pragma unroll
    for (int k = 0; k < M; k++) cq[k] = (T)0;
    if (order == 2) {
#pragma unroll
        for (int p = 0; p < MW; p++) {
            const int lim = (mthlim >> (8 * p)) & 0xff;
            if (lim == 0) continue;
            T wn2 = (T)0;
#pragma unroll
            for (int k = 0; k < M; k++)
                if (RP::template wnz<IXY>(p, k)) wn2 = wn2 + W[p * M + k] * W[p * M + k];
            if (eq0(wn2)) continue;
            T dot = (T)0;
            if (gt0(s[p])) {
#pragma unroll
                for (int k = 0; k < M; k++)
                    if (RP::template wnz<IXY>(p, k)) dot = dot + Wl[p * M + k] * W[p * M + k];
            } else {
#pragma unroll
                for (int k = 0; k < M; k++)
                    if (RP::template wnz<IXY>(p, k)) dot = dot + W[p * M + k] * Wr[p * M + k];
            }
            T phi = (T)0;
            if (!le0(dot)) {
#ifdef GCLAW_STRICT
                const T th = dot / wn2;
#else
                const T th = dot * rcp_fast(wn2);
#endif
                phi = gt0(th) ? philim_pos<T>(lim, th) : philim<T>(lim, th);
            }
#pragma unroll
            for (int k = 0; k < M; k++) W[p * M + k] = phi * W[p * M + k];
        }
        const T dtave = (T)0.5 * (dtdn + dtdn);
#pragma unroll
        for (int k = 0; k < M; k++) {
            T c = (T)0;
#pragma unroll
            for (int p = 0; p < MW; p++) {
                if (!RP::template wnz<IXY>(p, k)) continue;
                const T sa = tabs(s[p]);
                c = c + sa * ((T)1 - sa * dtave) * W[p * M + k];
            }
            cq[k] = c;
        }
    }
#pragma unroll
    for (int k = 0; k < M; k++) fa[k] = (T)0 + (T)0.5 * cq[k];
}

// phase_accum without transverse terms for one cell: apl = A+dQ of its left
// edge, amr = A-dQ of its right edge, fl / fr the correction fluxes of the
// two edges; q0 is the state the sweep starts from, overwritten with the
// new one.  The transverse terms of phase_accum are exact +0 here: they
// leave the sequence ((v + 0) + qo) - dt/dn fo (and, in the product FP64
// build, v - dt/dn s1).
template <int M, typename T>
__device__ __forceinline__ void update2(double *q0, const T *apl, const T *amr, const T *fl,
                                        const T *fr, T dtdn) {
    constexpr bool F64 = sizeof(T) == 8;
#pragma unroll
    for (int k = 0; k < M; k++) {
        T v = F64 ? (T)q0[k] : (T)0;
#ifndef GCLAW_STRICT
        if (F64) {
            const T s1 = (apl[k] + amr[k]) + (fr[k] - fl[k]);
            v = v - dtdn * s1;
            q0[k] = (double)v;
            continue;
        }
#endif
        const T qo = ((T)0 - dtdn * apl[k]) - dtdn * amr[k];
        const T fo = fr[k] - fl[k];
        v = ((v + (T)0) + qo) - dtdn * fo;
        q0[k] = F64 ? (double)v : q0[k] + f2d_bits((float)v);
    }
}

// block max of |s| and OR of the flag, one atomic each into the sweep's
// slot; the y-sweep's last block then finishes the step
template <typename T>
__device__ __forceinline__ void reduce2(const StepArgs &a, int slot, T smax, bool bad,
                                        bool finish, double dt) {
    __shared__ T s_red[NTP / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) smax = tmax(smax, __shfl_xor_sync(0xffffffffu, smax, off));
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = smax;
    const int any = __syncthreads_or(bad ? 1 : 0);
    if (threadIdx.x == 0) {
        for (int w = 1; w < NTP / 32; w++) smax = tmax(smax, s_red[w]);
        gclaw_ctrl *c = a.ctrl;
        atomicMax(&c->smax_bits[slot], (unsigned long long)__double_as_longlong((double)smax));
        if (any) atomicOr(&c->flags, 1u);
        if (finish) {
            __threadfence();
            if (atomicAdd(&c->blocks_done, 1u) == gridDim.x - 1) {
                __threadfence();
                finish_step(c, a.ctrl_mode, dt, dt / a.dx, dt / a.dy);
            }
        }
    }
}

// ---- warp windows along the sweep (x: rows; y: columns) --------------------
// Warp w takes line w mod (lines) -- consecutive warps on neighbouring lines,
// so that in the y-sweep the warps of a block share the cache sectors of
// their rows -- and P2_NWX windows of that line in a row.
template <template <typename> class RPT, typename T, int IXY>
__global__ void __launch_bounds__(NTP) p2_sweep_w(const StepArgs a, const typename RPT<T>::Params P,
                                                  Divisor dline, long long nwarps) {
    using RP = RPT<T>;
    constexpr int M = RP::M, MW = RP::MW, NA = RP::NA > 0 ? RP::NA : 1;
    constexpr unsigned FULL = 0xffffffffu;
    const Launch2<T> L = launch2<T>(a, IXY == 1 ? a.dx : a.dy);
    if (L.skip) return;
    const double *__restrict__ qin = L.par ? a.qin[1] : a.qin[0];
    double *qout = L.par ? a.qout[1] : a.qout[0];
    const T dtdn = L.dtdn;
    T smax = (T)0;
    bool bad = false;
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * NTP + threadIdx.x) >> 5;
    if (w < nwarps) {  // whole warps
        const unsigned grp = udiv((unsigned)w, dline);
        const int nl = IXY == 1 ? a.my : a.mx;  // lines across the sweep
        const int line = (int)((unsigned)w - grp * (unsigned)nl);
        const int n = IXY == 1 ? a.mx : a.my;
#pragma unroll 1
        for (int wi = 0; wi < P2_NWX; wi++) {
            const int c0 = ((int)grp * P2_NWX + wi) * P2_WIN;
            if (c0 >= n) break;
            const int x = c0 - 2 + lane;  // this lane's cell, and edge x on its left
            T q[M], ql[M], aux[NA], al[NA];
            if (IXY == 1) load_cell2<M, 1, T>(a, qin, min(x, n + 1), line, q);
            else load_cell2<M, 2, T>(a, qin, line, min(x, n + 1), q);
            if (RP::NA > 0) RP::cell_aux(P, q, aux);
#pragma unroll
            for (int k = 0; k < M; k++) ql[k] = __shfl_up_sync(FULL, q[k], 1);
#pragma unroll
            for (int f = 0; f < RP::NA; f++) al[f] = __shfl_up_sync(FULL, aux[f], 1);
            T W[MW * M], s[MW], am[M], ap[M];
            T sm = (T)0;
            bool bd = false;
            solve2<RP, IXY, T>(P, x, n, ql, al, q, aux, W, s, am, ap, sm, bd);
            if (lane >= 1 && x <= n + 1) {  // edges -1 .. n + 1
                smax = tmax(smax, sm);
                bad |= bd;
            }
            // the upwind neighbour's unlimited wave of each family
            T Wn[MW * M];
#pragma unroll
            for (int p = 0; p < MW; p++) {
                const int from = (gt0(s[p]) ? lane - 1 : lane + 1) & 31;
#pragma unroll
                for (int k = 0; k < M; k++)
                    Wn[p * M + k] = RP::template wnz<IXY>(p, k)
                                        ? __shfl_sync(FULL, W[p * M + k], from)
                                        : (T)0;
            }
            T fa[M], amr[M], far[M];
            limit2<RP, IXY, T>(a.mthlim, a.order, Wn, W, Wn, s, dtdn, fa);
#pragma unroll
            for (int k = 0; k < M; k++) {
                amr[k] = __shfl_down_sync(FULL, am[k], 1);
                far[k] = __shfl_down_sync(FULL, fa[k], 1);
            }
            if (lane >= 2 && lane < 2 + P2_WIN && x < n) {
                const size_t o = IXY == 1 ? (size_t)M * ((size_t)x + (size_t)a.mx * (size_t)line)
                                          : (size_t)M * ((size_t)line + (size_t)a.mx * (size_t)x);
                double q0[M];
                load_row<M>(qin, o, q0);
                update2<M, T>(q0, ap, amr, fa, far, dtdn);
                store_row<M>(qout, o, q0);
            }
        }
    }
    reduce2<T>(a, IXY - 1, smax, bad, IXY == 2 && !a.no_finish, L.dt);
}

// ---- y-sweep: marching columns ----------------------------------------------
template <template <typename> class RPT, typename T>
__global__ void __launch_bounds__(NTP, ycol_blocks<RPT, T>())
    p2_sweep_y(const StepArgs a, const typename RPT<T>::Params P, Divisor dcol, long long nthr) {
    using RP = RPT<T>;
    constexpr int M = RP::M, MW = RP::MW, NA = RP::NA > 0 ? RP::NA : 1;
    constexpr int PL = ycol_len<T>();
    const Launch2<T> L = launch2<T>(a, a.dy);
    if (L.skip) return;
    const double *__restrict__ qin = L.par ? a.qin[1] : a.qin[0];
    double *qout = L.par ? a.qout[1] : a.qout[0];
    const T dtdn = L.dtdn;
    T smax = (T)0;
    bool bad = false;
    const long long t = (long long)blockIdx.x * NTP + threadIdx.x;
    if (t < nthr) {
        const unsigned ch = udiv((unsigned)t, dcol);
        const int i = (int)((unsigned)t - ch * (unsigned)a.mx);
        const int n = a.my;
        const int c0 = (int)ch * PL, c1 = min(c0 + PL, n);
        auto load = [&](int c, T *q, T *aux) {
            load_cell2<M, 2, T>(a, qin, i, c, q);
            if (RP::NA > 0) RP::cell_aux(P, q, aux);
        };
        T qa[M], qb[M], xa[NA], xb[NA], am[M], ap[M];
        T Wp[MW * M], Wc[MW * M], Wn[MW * M], Wx[MW * M];
        T sc[MW], sn[MW], sx[MW];
        T apc[M], amn[M], apn[M], fa0[M], fa1[M];
        load(c0 - 2, qa, xa);
        load(c0 - 1, qb, xb);
        solve2<RP, 2, T>(P, c0 - 1, n, qa, xa, qb, xb, Wp, sx, am, ap, smax, bad);
        load(c0, qa, xa);
        solve2<RP, 2, T>(P, c0, n, qb, xb, qa, xa, Wc, sc, am, apc, smax, bad);
        load(c0 + 1, qb, xb);
        solve2<RP, 2, T>(P, c0 + 1, n, qa, xa, qb, xb, Wn, sn, amn, apn, smax, bad);
        limit2<RP, 2, T>(a.mthlim, a.order, Wp, Wc, Wn, sc, dtdn, fa0);
        // qb holds the cell after the current one; the one after that is
        // loaded an iteration ahead
        T qf[M];
        load_cell2<M, 2, T>(a, qin, i, c0 + 2, qf);
#pragma unroll 1
        for (int c = c0; c < c1; c++) {
#pragma unroll
            for (int k = 0; k < M; k++) qa[k] = qf[k];
            if (c + 1 < c1) load_cell2<M, 2, T>(a, qin, i, c + 3, qf);
            if (RP::NA > 0) RP::cell_aux(P, qa, xa);
            solve2<RP, 2, T>(P, c + 2, n, qb, xb, qa, xa, Wx, sx, am, ap, smax, bad);
            limit2<RP, 2, T>(a.mthlim, a.order, Wc, Wn, Wx, sn, dtdn, fa1);
            const size_t o = (size_t)M * ((size_t)i + (size_t)a.mx * (size_t)c);
            double q0[M];
            load_row<M>(qin, o, q0);
            update2<M, T>(q0, apc, amn, fa0, fa1, dtdn);
            store_row<M>(qout, o, q0);
#pragma unroll
            for (int f = 0; f < MW * M; f++) {
                Wc[f] = Wn[f];
                Wn[f] = Wx[f];
            }
#pragma unroll
            for (int p = 0; p < MW; p++) sn[p] = sx[p];
#pragma unroll
            for (int k = 0; k < M; k++) {
                apc[k] = apn[k];
                amn[k] = am[k];
                apn[k] = ap[k];
                fa0[k] = fa1[k];
                qb[k] = qa[k];
            }
#pragma unroll
            for (int f = 0; f < RP::NA; f++) xb[f] = xa[f];
        }
    }
    reduce2<T>(a, 1, smax, bad, !a.no_finish, L.dt);
}

// The two sweeps of one split step: x from qin[par] into qtmp (ax), y from
// qtmp into qout[par] (ay), whose last block finishes the step.  Returns
// GCLAW_ERR_UNSUPPORTED when the grid is beyond the kernels' 32-bit
// thread numbering (the caller then runs the tile kernels).
template <template <typename> class RPT, typename T>
static int split_step(const gclaw_solver *s, const StepArgs &ax, const StepArgs &ay,
                      cudaStream_t st, bool y_windows) {
    constexpr int PL = ycol_len<T>();
    constexpr int WW = P2_WIN * P2_NWX;
    const long long nwarps = (long long)s->my * ((s->mx + WW - 1) / WW);
    const long long nwarps_y = (long long)s->mx * ((s->my + WW - 1) / WW);
    const long long nthr = (long long)s->mx * ((s->my + PL - 1) / PL);
    if (nwarps * 32 >= (1ll << 31) || nwarps_y * 32 >= (1ll << 31) || nthr >= (1ll << 31))
        return GCLAW_ERR_UNSUPPORTED;
    const typename RPT<T>::Params P = RPT<T>::make(s->problem_data);
    const unsigned bx = (unsigned)((nwarps * 32 + NTP - 1) / NTP);
    p2_sweep_w<RPT, T, 1><<<bx, NTP, 0, st>>>(ax, P, make_divisor(s->my), nwarps);
    if (y_windows) {
        const unsigned by = (unsigned)((nwarps_y * 32 + NTP - 1) / NTP);
        p2_sweep_w<RPT, T, 2><<<by, NTP, 0, st>>>(ay, P, make_divisor(s->mx), nwarps_y);
    } else {
        const unsigned by = (unsigned)((nthr + NTP - 1) / NTP);
        p2_sweep_y<RPT, T><<<by, NTP, 0, st>>>(ay, P, make_divisor(s->mx), nthr);
    }
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

}  // namespace p2
}  // namespace gclaw
