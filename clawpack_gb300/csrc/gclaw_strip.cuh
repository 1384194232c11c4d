// gclaw_strip.cuh -- FP32-bulk classic step with register-resident strips.
//
// The tile kernel (gclaw_step_impl.cuh) stages a 2D tile in shared memory
// and runs the step in barrier-separated phases; in FP32 it is bound by
// instruction issue, with shared-memory traffic (about 280 accesses per
// cell-update) and barrier waits as the largest overheads.  This kernel maps
// the same step onto warps that march up the grid instead:
//
//   * a warp owns a strip of 28 output columns: lane L holds column
//     i0 + L - 2, lanes 0-1 and 30-31 are the halo the limiter and the
//     transverse terms need, and the warp walks rows j0-2 .. j1+1 of its
//     row segment [j0, j1);
//   * x-edges: lane L solves the Riemann problem on its left edge with the
//     left cell's state taken from lane L-1 by a shuffle; the limiter's
//     upwind wave and the right edge's contributions come from the
//     neighbouring lanes the same way;
//   * y-edges: each lane keeps the last three y-edge records of its column
//     in registers, so the limiter and the correction flux of edge r-3/2
//     are available when row r has been read; the transverse parts that
//     go to the neighbouring columns are exchanged by shuffles;
//   * per cell, the increments are summed in a four-row register window in
//     the order of the tile kernel (x-sweep: slice before, own slice,
//     slice after; then the y-sweep the same way), and row r-2 is written
//     once as q_old + increment.
//
// No shared memory and no barrier is used until the block-wide Courant
// number reduction at the end.  The Riemann solvers, the limiter and the
// per-cell aux are the tile kernel's device functions, and the conversions
// and expressions are the same, so the results equal the tile kernel's in
// value up to multiply-add contraction choices.
#pragma once

#include "gclaw_step_impl.cuh"

namespace gclaw {

constexpr int STRIP_W = 28;      // output columns per warp
#ifndef GCLAW_STRIP_NW
#define GCLAW_STRIP_NW 4
#endif
constexpr int STRIP_NW = GCLAW_STRIP_NW;  // warps per block
constexpr int STRIP_MIN_ROWS = 16;

// Resident blocks per SM the kernel is compiled for (the register budget):
// acoustics and shallow water fit 128 registers, Euler gets 168.
// RING: keep the y-edge records and the saved limited-edge terms in this
// warp's shared memory (three slots rotating with the rows, lane-fastest,
// each lane touching only its own column's slots) instead of registers, for
// solvers whose records would not leave room for enough resident warps.
// MINB64: the same for the FP64 kernel, which always uses the ring.
template <template <typename> class RPT>
struct StripCfg {
    static constexpr int MINB = 3, MINB64 = 2;
    static constexpr bool RING = true;
};
template <>
struct StripCfg<RpAcoustics> {
    static constexpr int MINB = 4, MINB64 = 2;
    static constexpr bool RING = false;
};
template <>
struct StripCfg<RpShallow> {
    static constexpr int MINB = 4, MINB64 = 2;  // FP32: 127 registers with the ring, no spills
    static constexpr bool RING = true;
};
template <template <typename> class RPT, typename T>
__host__ __device__ constexpr bool strip_ring() {
    return sizeof(T) == 8 || StripCfg<RPT>::RING;
}
template <template <typename> class RPT, typename T>
__host__ __device__ constexpr int strip_minb() {
    return sizeof(T) == 8 ? StripCfg<RPT>::MINB64 : StripCfg<RPT>::MINB;
}

// Real type of a solver instance RpX<T>.
template <class RP>
struct rp_real;
template <template <typename> class R, typename T>
struct rp_real<R<T>> {
    using type = T;
};

// Elements (of the solver's real type) of shared memory per lane for the
// y-edge ring of solver RP.
template <class RP>
__host__ __device__ constexpr int strip_ring_floats() {
    return 3 * (RP::MW * RP::M + RP::MW + 2 * RP::M + (RP::NR > 0 ? RP::NR : 1)) + 4 * RP::M;
}

template <typename T>
__device__ __forceinline__ T shfl_up1(T v) {
    return __shfl_up_sync(0xffffffffu, v, 1);
}
template <typename T>
__device__ __forceinline__ T shfl_dn1(T v) {
    return __shfl_down_sync(0xffffffffu, v, 1);
}

// Limiter, correction flux and transverse splitting of one edge (the body
// of phase_limit for a single edge, with the same expressions and tests).
// W is limited in place; wu_lo / wu_hi are the waves of the edge below /
// above along the sweep (only the components the solver can make nonzero
// are read).
template <class RP, int IXY, typename T>
__device__ __forceinline__ void strip_limit_edge(const typename RP::Params &P, T *W, const T *s,
                                                 const T *wu_lo, const T *wu_hi, const T *am,
                                                 const T *ap, const T *R, int mthlim, int order,
                                                 int tw, T dtdn, T *fa, T *bmm, T *bpm, T *bmp,
                                                 T *bpp) {
    constexpr int M = RP::M, MW = RP::MW;
    T cq[M];
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
                    if (RP::template wnz<IXY>(p, k)) dot = dot + wu_lo[p * M + k] * W[p * M + k];
            } else {
#pragma unroll
                for (int k = 0; k < M; k++)
                    if (RP::template wnz<IXY>(p, k)) dot = dot + W[p * M + k] * wu_hi[p * M + k];
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
                if constexpr (RP::FWAVE)  // sign(s) (1 - |s| dt/dx) Z
                    c = c + sign_times((T)1 - sa * dtave, s[p]) * W[p * M + k];
                else
                    c = c + sa * ((T)1 - sa * dtave) * W[p * M + k];
            }
            cq[k] = c;
        }
    }
#pragma unroll
    for (int k = 0; k < M; k++) fa[k] = (T)0 + (T)0.5 * cq[k];
    if (tw > 0) {
        T amf[M], apf[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            amf[k] = am[k];
            apf[k] = ap[k];
        }
        if (order == 2 && tw == 2) {
#pragma unroll
            for (int k = 0; k < M; k++) {
                amf[k] = amf[k] + cq[k];
                apf[k] = apf[k] - cq[k];
            }
        }
        RP::template rpt2<IXY>(P, R, amf, bmm, bpm);
        RP::template rpt2<IXY>(P, R, apf, bmp, bpp);
    } else {
#pragma unroll
        for (int k = 0; k < M; k++) bmm[k] = bpm[k] = bmp[k] = bpp[k] = (T)0;
    }
}

// One y-edge record between rows.
template <class RP>
struct StripEdge {
    using T = typename rp_real<RP>::type;
    T W[RP::MW * RP::M], s[RP::MW], am[RP::M], ap[RP::M], R[RP::NR > 0 ? RP::NR : 1];
};

template <class RP>
__device__ __forceinline__ void load_row(const StepArgs &a, const double *__restrict__ qin, int c,
                                         int r, double *qd) {
#pragma unroll
    for (int k = 0; k < RP::M; k++) qd[k] = load_q<RP::M>(a, qin, k, c, r);
}

// y-edge records in a warp's shared-memory ring: slot-major, field, lane.
template <class RP>
struct StripRing {
    using T = typename rp_real<RP>::type;
    static constexpr int NW = RP::MW * RP::M, NR = RP::NR > 0 ? RP::NR : 1;
    static constexpr int NF = NW + RP::MW + 2 * RP::M + NR;
    T *base;  // this warp's area, lane-offset applied
    __device__ __forceinline__ T &at(int slot, int f) const { return base[(slot * NF + f) * 32]; }
    __device__ __forceinline__ T &lim(int f) const { return base[(3 * NF + f) * 32]; }
    __device__ __forceinline__ void put(int slot, const StripEdge<RP> &e) const {
#pragma unroll
        for (int f = 0; f < NW; f++)
            if (RP::template wnz<2>(f / RP::M, f % RP::M)) at(slot, f) = e.W[f];
#pragma unroll
        for (int p = 0; p < RP::MW; p++) at(slot, NW + p) = e.s[p];
#pragma unroll
        for (int k = 0; k < RP::M; k++) {
            at(slot, NW + RP::MW + k) = e.am[k];
            at(slot, NW + RP::MW + RP::M + k) = e.ap[k];
        }
#pragma unroll
        for (int r = 0; r < NR; r++) at(slot, NW + RP::MW + 2 * RP::M + r) = e.R[r];
    }
    __device__ __forceinline__ void get(int slot, StripEdge<RP> &e) const {
#pragma unroll
        for (int f = 0; f < NW; f++)
            e.W[f] = RP::template wnz<2>(f / RP::M, f % RP::M) ? at(slot, f) : (T)0;
#pragma unroll
        for (int p = 0; p < RP::MW; p++) e.s[p] = at(slot, NW + p);
#pragma unroll
        for (int k = 0; k < RP::M; k++) {
            e.am[k] = at(slot, NW + RP::MW + k);
            e.ap[k] = at(slot, NW + RP::MW + RP::M + k);
        }
#pragma unroll
        for (int r = 0; r < NR; r++) e.R[r] = at(slot, NW + RP::MW + 2 * RP::M + r);
    }
    __device__ __forceinline__ void get_w(int slot, T *W) const {
#pragma unroll
        for (int f = 0; f < NW; f++)
            W[f] = RP::template wnz<2>(f / RP::M, f % RP::M) ? at(slot, f) : (T)0;
    }
};

// The march of one warp over rows [j0, j1) of its strip.  T is the
// arithmetic type: float for FP32-bulk (the window holds increments added to
// the FP64 state at the end), double for FP64 (the window holds the state
// itself, each row starting from q in the tile kernel's order, so the
// -fmad=false build reproduces the oracle).  ring: this warp's shared-memory
// area (strip_ring_floats elements of T per lane) when RING.
template <template <typename> class RPT, typename T, bool RING>
__device__ __forceinline__ void strip_run(const StepArgs &a, const typename RPT<T>::Params &P,
                                          const double *__restrict__ qin,
                                          double *__restrict__ qout, T dtdx, T dtdy, int lane,
                                          int c, int j0, int j1, T &smax_x, T &smax_y, bool &bad,
                                          T *ring) {
    using RP = RPT<T>;
    constexpr bool F64 = sizeof(T) == 8;
    const StripRing<RP> yr{ring + lane};
    int so = 0, sm = 1, sn = 2;  // ring slots of the y-edges r-5/2, r-3/2, r-1/2
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR > 0 ? RP::NR : 1;
    constexpr int NA = RP::NA > 0 ? RP::NA : 1;
    const int mthlim = a.mthlim, order = a.order, tw = a.tw;
    const int mx = a.mx, my = a.my;
    const T hx = (T)0.5 * dtdx, hy = (T)0.5 * dtdy;

    // Courant-number ownership: every x-edge (edge index c in [0, mx]) of
    // rows -1..my and every y-edge of columns -1..mx is counted by one
    // strip (a column at lane 30 may be counted twice, harmless for a max).
    const bool own = lane >= 2 && lane <= 29;
    const bool cfl_xcol = c >= 0 && c <= mx && (own || (c == mx && lane == 30));
    const bool cfl_ycol =
        c >= -1 && c <= mx && (own || (c == -1 && lane == 1) || (c == mx && lane == 30));
    const bool out_col = own && c < mx;
    const int onx = a.ghosted ? mx + 4 : mx, ooff = a.ghosted ? 2 : 0;

    T qp[M], ap_[NA];   // row r-1 and its aux
    T qc[M], ac[NA];    // row r
    StripEdge<RP> Eo, Em;  // y-edges r-5/2 (W, s used) and r-3/2
    T A0[M], A1[M], A2[M], A3[M];  // rows r-2 .. r+1 (increments, or states in FP64)
    T LAP[M], LFA[M], LBMP[M], LBPP[M];  // limited y-edge j-1/2 of the output row j
#pragma unroll
    for (int k = 0; k < M; k++) A0[k] = A1[k] = A2[k] = A3[k] = (T)0;
#pragma unroll
    for (int k = 0; k < M; k++) LAP[k] = LFA[k] = LBMP[k] = LBPP[k] = qp[k] = (T)0;
#pragma unroll
    for (int f = 0; f < NA; f++) ap_[f] = (T)0;
    Em = StripEdge<RP>{};
    Eo = Em;

    // FP32: row r+1 is loaded during row r.  FP64: rows are loaded two ahead,
    // because the accumulator of row r+2 starts from its state at the end of
    // row r.
    double qn[M], qf[M];
    load_row<RP>(a, qin, c, j0 - 2, qn);
    if constexpr (F64) load_row<RP>(a, qin, c, j0 - 1, qf);
    for (int r = j0 - 2; r <= j1 + 1; r++) {
#pragma unroll
        for (int k = 0; k < M; k++) qc[k] = from_double<T>(qn[k]);
        if constexpr (F64) {
#pragma unroll
            for (int k = 0; k < M; k++) qn[k] = qf[k];
            if (r + 2 <= j1 + 1) load_row<RP>(a, qin, c, r + 2, qf);  // in flight
        } else {
            if (r <= j1) load_row<RP>(a, qin, c, r + 1, qn);  // in flight during this row
        }
        RP::cell_aux(P, qc, ac);

        // ---- x-sweep of row r -------------------------------------------------
        if (r >= j0 - 1 && r <= j1) {
            T ql[M], al[NA];
#pragma unroll
            for (int k = 0; k < M; k++) ql[k] = shfl_up1(qc[k]);
#pragma unroll
            for (int f = 0; f < NA; f++) al[f] = shfl_up1(ac[f]);
            T W[MW * M], s[MW], am[M], apx[M], R[NR];
            const bool eb = RP::template rpn2<1>(P, ql, qc, al, ac, W, s, am, apx, R);
            const bool cnt_row = (r >= j0 && r < j1) || r == -1 || r == my;
            if (cfl_xcol && cnt_row) {
                bad |= eb;
#pragma unroll
                for (int p = 0; p < MW; p++) {
                    bad |= isnan_v(s[p]);
                    smax_x = max_abs(smax_x, s[p]);
                }
            }
            // upwind waves of the neighbouring edges (lanes L-1, L+1)
            T wlo[MW * M], whi[MW * M];
#pragma unroll
            for (int f = 0; f < MW * M; f++) {
                if (RP::template wnz<1>(f / M, f % M)) {
                    wlo[f] = shfl_up1(W[f]);
                    whi[f] = shfl_dn1(W[f]);
                } else {
                    wlo[f] = whi[f] = (T)0;
                }
            }
            T fa[M], bmm[M], bpm[M], bmp[M], bpp[M];
            strip_limit_edge<RP, 1>(P, W, s, wlo, whi, am, apx, R, mthlim, order, tw, dtdx, fa,
                                    bmm, bpm, bmp, bpp);
            // contributions of the right edge (lane L+1) to this cell
#pragma unroll
            for (int k = 0; k < M; k++) {
                const T amn = shfl_dn1(am[k]), fan = shfl_dn1(fa[k]);
                const T bmmn = shfl_dn1(bmm[k]), bpmn = shfl_dn1(bpm[k]);
                const T qo = ((T)0 - dtdx * apx[k]) - dtdx * amn;
                const T fo = fan - fa[k];
                const T g1 = ((T)0 - hx * bmmn) - hx * bmp[k];
                const T g2 = ((T)0 - hx * bpmn) - hx * bpp[k];
                A1[k] = A1[k] - dtdy * g1;                                  // slice after
                A2[k] = ((A2[k] + qo) - dtdx * fo) - dtdy * (g2 - g1);      // own slice
                A3[k] = A3[k] + dtdy * g2;                                  // slice before
            }
        }

        // ---- y-sweep: edge r-1/2, limiting of edge r-3/2, row r-2 ------------
        if (r >= j0 - 1) {
            StripEdge<RP> En;
            const bool eb = RP::template rpn2<2>(P, qp, qc, ap_, ac, En.W, En.s, En.am, En.ap,
                                                 En.R);
            const bool cnt_row = (r >= j0 && r < j1) || r == my;
            if (cfl_ycol && cnt_row) {
                bad |= eb;
#pragma unroll
                for (int p = 0; p < MW; p++) {
                    bad |= isnan_v(En.s[p]);
                    smax_y = max_abs(smax_y, En.s[p]);
                }
            }
            if (r >= j0 + 1) {
                if constexpr (RING) {
                    yr.get(sm, Em);
                    yr.get_w(so, Eo.W);
#pragma unroll
                    for (int k = 0; k < M; k++) {
                        LAP[k] = yr.lim(k);
                        LFA[k] = yr.lim(M + k);
                        LBMP[k] = yr.lim(2 * M + k);
                        LBPP[k] = yr.lim(3 * M + k);
                    }
                }
                T W[MW * M];
#pragma unroll
                for (int f = 0; f < MW * M; f++) W[f] = Em.W[f];
                T fa[M], bmm[M], bpm[M], bmp[M], bpp[M];
                strip_limit_edge<RP, 2>(P, W, Em.s, Eo.W, En.W, Em.am, Em.ap, Em.R, mthlim, order,
                                        tw, dtdy, fa, bmm, bpm, bmp, bpp);
                if (r >= j0 + 2) {
                    // row j = r-2: edges j-1/2 (saved) and j+1/2 (this one)
                    T g1o[M], g2o[M];
#pragma unroll
                    for (int k = 0; k < M; k++) {
                        g1o[k] = ((T)0 - hy * bmm[k]) - hy * LBMP[k];
                        g2o[k] = ((T)0 - hy * bpm[k]) - hy * LBPP[k];
                    }
#pragma unroll
                    for (int k = 0; k < M; k++) {
                        const T g2b = shfl_up1(g2o[k]);   // column c-1, slice before
                        const T g1a = shfl_dn1(g1o[k]);   // column c+1, slice after
                        const T qo = ((T)0 - dtdy * LAP[k]) - dtdy * Em.am[k];
                        const T fo = fa[k] - LFA[k];
                        T v = A0[k];
                        v = v + dtdx * g2b;
                        v = ((v + qo) - dtdy * fo) - dtdx * (g2o[k] - g1o[k]);
                        v = v - dtdx * g1a;
                        A0[k] = v;
                    }
                    if (out_col) {
                        const int j = r - 2;
                        const size_t o =
                            (size_t)M * ((size_t)(c + ooff) + (size_t)onx * (size_t)(j + ooff));
#pragma unroll
                        for (int k = 0; k < M; k++) {
                            if constexpr (F64) qout[o + k] = (double)A0[k];
                            else qout[o + k] = __ldg(qin + o + k) + f2d_bits((float)A0[k]);
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < M; k++) {
                    LAP[k] = Em.ap[k];
                    LFA[k] = fa[k];
                    LBMP[k] = bmp[k];
                    LBPP[k] = bpp[k];
                    if constexpr (RING) {
                        yr.lim(k) = LAP[k];
                        yr.lim(M + k) = LFA[k];
                        yr.lim(2 * M + k) = LBMP[k];
                        yr.lim(3 * M + k) = LBPP[k];
                    }
                }
            }
            if constexpr (RING) {
                yr.put(sn, En);
                const int t = so;
                so = sm;
                sm = sn;
                sn = t;
            } else {
                Eo = Em;
                Em = En;
            }
        }

        // ---- shift the row windows ---------------------------------------------
#pragma unroll
        for (int k = 0; k < M; k++) {
            qp[k] = qc[k];
            A0[k] = A1[k];
            A1[k] = A2[k];
            A2[k] = A3[k];
            A3[k] = F64 ? (T)qf[k] : (T)0;  // FP64: row r+2 starts from its state
        }
#pragma unroll
        for (int f = 0; f < NA; f++) ap_[f] = ac[f];
    }
}

}  // namespace gclaw
