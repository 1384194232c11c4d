// gclaw_adjoint.cu -- hand-written adjoint (reverse mode) of one classic
// unsplit 2D step, for gradients through time stepping.
//
// With q_new = step(q_old) at a fixed dt, gclaw_adjoint_step computes
//   lam_old = (d q_new / d q_old)^T lam_new
// for acoustics_2D and shallow_roe_with_efix_2D, in FP64 or FP32 (the
// FP32-bulk arithmetic; lam is stored in FP64).  One CTA per tile:
//   1. recompute the forward for the tile and its halo: load with boundary
//      conditions, per-cell aux values, normal Riemann problems (rpn2);
//   2. per sweep, adjoints of every edge output (fluctuations, correction
//      flux, transverse terms) from lam_new of the tile's own cells -- the
//      transpose of the per-cell update of the forward;
//   3. per edge, recompute limiter / correction flux / folded fluctuations
//      and run their reverse (rpt2_adj, the correction flux, the limiter,
//      whose upwind-neighbour term goes to that neighbour edge's slot);
//   4. per edge, rpn2_adj (with the entropy fix) and the per-cell aux
//      reverse give the adjoints of the two cells of the edge; they are
//      summed per cell in shared memory in a fixed order;
//   5. the tile's halo sums are mapped back through the boundary conditions
//      (ghost cell -> source cell, sign flip of the normal momentum at walls)
//      and added to lam_old with atomics.
// Each tile handles the (edge -> output cell) pairs whose output cell it
// owns, so the sums over tiles are the full transpose.  Branches are taken
// as the forward takes them on the same state.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gclaw.h"
#include "gclaw_adjoint.cuh"
#include "gclaw_step_impl.cuh"

namespace gclaw {

template <class RP, class AD, int TX, int TY>
struct AdjTile {
    using TL = Tile<RP, TX, TY>;
    static constexpr int M = RP::M, MW = RP::MW;
    static constexpr int NA = RP::NA > 0 ? RP::NA : 1;
    static constexpr int NR = RP::NR > 0 ? RP::NR : 1;
    static constexpr int QN = TL::QN, NE1 = TL::NE1;
    // forward edge records with every wave component: W[MW*M], s[MW],
    // amdq[M], apdq[M], Roe state[NR]
    static constexpr int FW = 0, FS = MW * M, FAM = FS + MW, FAP = FAM + M, FR = FAP + M;
    static constexpr int EAW = FR + RP::NR;
    // adjoint slots per edge: own W, s, amdq, apdq, Roe state, and W from
    // the left / right neighbour edge's limiter
    static constexpr int GW = 0, GS = MW * M, GAM = GS + MW, GAP = GAM + M, GR = GAP + M;
    static constexpr int GWL = GR + NR, GWR = GWL + MW * M, GBW = GWR + MW * M;
    template <typename T>
    static constexpr size_t smem_bytes() {
        return sizeof(T) * ((size_t)M * QN + (size_t)NA * QN + (size_t)EAW * NE1 +
                            (size_t)GBW * NE1 + (size_t)M * TX * TY + (size_t)M * QN);
    }
};

// lam of tile cell (x, y) in tile-local coordinates, 0 outside the tile
template <typename T, int TX, int TY>
__device__ __forceinline__ T lam_at(const T *LT, int k, int x, int y) {
    return (x >= 0 && x < TX && y >= 0 && y < TY) ? LT[(k * TY + y) * TX + x] : (T)0;
}

template <class RP, class AD, typename T, int IXY, int TX, int TY, int NT>
__device__ __forceinline__ void adj_sweep(const StepArgs &a, const typename RP::Params &P,
                                          const T *QS, const T *CA, T *EA, T *GB, const T *LT,
                                          T *LA, int i0, int j0, T dtdn, T dtdt) {
    using TL = Tile<RP, TX, TY>;
    using AT = AdjTile<RP, AD, TX, TY>;
    using SI = SweepIdx<IXY, TX, TY>;
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR, NA = RP::NA;
    constexpr int NA1 = SI::NA, NS = SI::NS, NA2 = SI::NA2, STEP = SI::STEP1;
    constexpr int ANA = AT::NA, ANR = AT::NR;
    (void)i0;
    (void)j0;

    // F1: forward Riemann problems of every edge, zeroed adjoint slots
    for (int it = threadIdx.x; it < NA1 * NS; it += NT) {
        int ea, sl;
        SI::split1(it, ea, sl);
        const int cl = (IXY == 1) ? (sl + 1) * TL::QW + ea : ea * TL::QW + sl + 1;
        const int cr = cl + ((IXY == 1) ? 1 : TL::QW);
        T ql[M], qr[M], al[ANA], ar[ANA];
#pragma unroll
        for (int k = 0; k < M; k++) {
            ql[k] = QS[k * TL::QN + cl];
            qr[k] = QS[k * TL::QN + cr];
        }
#pragma unroll
        for (int f = 0; f < NA; f++) {
            al[f] = CA[f * TL::QN + cl];
            ar[f] = CA[f * TL::QN + cr];
        }
        T W[MW * M], s[MW], am[M], ap[M], R[ANR];
        RP::template rpn2<IXY>(P, ql, qr, al, ar, W, s, am, ap, R);
#pragma unroll
        for (int f = 0; f < MW * M; f++) EA[(AT::FW + f) * TL::NE1 + it] = W[f];
#pragma unroll
        for (int p = 0; p < MW; p++) EA[(AT::FS + p) * TL::NE1 + it] = s[p];
#pragma unroll
        for (int k = 0; k < M; k++) {
            EA[(AT::FAM + k) * TL::NE1 + it] = am[k];
            EA[(AT::FAP + k) * TL::NE1 + it] = ap[k];
        }
#pragma unroll
        for (int r = 0; r < NR; r++) EA[(AT::FR + r) * TL::NE1 + it] = R[r];
#pragma unroll 1
        for (int f = 0; f < AT::GBW; f++) GB[f * AT::NE1 + it] = (T)0;
    }
    __syncthreads();

    // B2/B3: edge-output adjoints from lam_new, then the reverse of rpt2, the
    // correction flux and the limiter
    const T h = (T)0.5 * dtdn;
    for (int it2 = threadIdx.x; it2 < NA2 * NS; it2 += NT) {
        int e2, sl;
        SI::split2(it2, e2, sl);
        const int ea = e2 + 1;
        const int ie = SI::item1(ea, sl);
        // tile-local cell coordinates: along the sweep the edge separates
        // cells ea-2 and ea-1; across it the slice is sl-1
        int xl, yl, xr, yr, tx, ty;  // left / right cell, transverse step
        if (IXY == 1) { xl = ea - 2; xr = ea - 1; yl = yr = sl - 1; tx = 0; ty = 1; }
        else { yl = ea - 2; yr = ea - 1; xl = xr = sl - 1; tx = 1; ty = 0; }
        T amb[M], apb[M], fab[M], bmmb[M], bpmb[M], bmpb[M], bppb[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            const T lr = lam_at<T, TX, TY>(LT, k, xr, yr), ll = lam_at<T, TX, TY>(LT, k, xl, yl);
            apb[k] = -dtdn * lr;
            amb[k] = -dtdn * ll;
            fab[k] = dtdn * (lr - ll);
            // transverse flux adjoints of the left / right cell (low and high
            // transverse edges): G1 = dtdt (lam(c) - lam(c-1)), G2 = dtdt (lam(c+1) - lam(c))
            const T g1l = dtdt * (ll - lam_at<T, TX, TY>(LT, k, xl - tx, yl - ty));
            const T g2l = dtdt * (lam_at<T, TX, TY>(LT, k, xl + tx, yl + ty) - ll);
            const T g1r = dtdt * (lr - lam_at<T, TX, TY>(LT, k, xr - tx, yr - ty));
            const T g2r = dtdt * (lam_at<T, TX, TY>(LT, k, xr + tx, yr + ty) - lr);
            bmmb[k] = -h * g1l;
            bpmb[k] = -h * g2l;
            bmpb[k] = -h * g1r;
            bppb[k] = -h * g2r;
        }
        // forward recompute of the limited waves and folded fluctuations
        T W[MW * M], s[MW], am[M], ap[M], R[ANR], cq[M];
#pragma unroll
        for (int f = 0; f < MW * M; f++) W[f] = EA[(AT::FW + f) * TL::NE1 + ie];
#pragma unroll
        for (int p = 0; p < MW; p++) s[p] = EA[(AT::FS + p) * TL::NE1 + ie];
#pragma unroll
        for (int k = 0; k < M; k++) {
            am[k] = EA[(AT::FAM + k) * TL::NE1 + ie];
            ap[k] = EA[(AT::FAP + k) * TL::NE1 + ie];
            cq[k] = (T)0;
        }
#pragma unroll
        for (int r = 0; r < NR; r++) R[r] = EA[(AT::FR + r) * TL::NE1 + ie];
        T phi[MW], theta[MW], wn2v[MW];
        int upd[MW];  // -1: upwind neighbour is the previous edge, +1: next, 0: not limited
        const T dtave = (T)0.5 * (dtdn + dtdn);
        if (a.order == 2) {
#pragma unroll
            for (int p = 0; p < MW; p++) {
                const int lim = (a.mthlim >> (8 * p)) & 0xff;
                phi[p] = (T)1;
                theta[p] = (T)0;
                upd[p] = 0;
                T wn2 = (T)0;
#pragma unroll
                for (int k = 0; k < M; k++) wn2 = wn2 + W[p * M + k] * W[p * M + k];
                wn2v[p] = wn2;
                if (lim == 0 || wn2 == (T)0) continue;
                const int nb = s[p] > (T)0 ? ie - STEP : ie + STEP;
                upd[p] = s[p] > (T)0 ? -1 : 1;
                T dot = (T)0;
#pragma unroll
                for (int k = 0; k < M; k++)
                    dot = dot + EA[(AT::FW + p * M + k) * TL::NE1 + nb] * W[p * M + k];
                theta[p] = dot / wn2;
                phi[p] = philim<T>(lim, theta[p]);
            }
#pragma unroll
            for (int k = 0; k < M; k++) {
                T c = (T)0;
#pragma unroll
                for (int p = 0; p < MW; p++) {
                    const T sa = tabs(s[p]);
                    c = c + sa * ((T)1 - sa * dtave) * (phi[p] * W[p * M + k]);
                }
                cq[k] = c;
            }
        }
        const bool fold = a.order == 2 && a.tw == 2;
        T amf[M], apf[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            amf[k] = fold ? am[k] + cq[k] : am[k];
            apf[k] = fold ? ap[k] - cq[k] : ap[k];
        }
        // reverse of the transverse splitting
        T asmb[M], aspb[M], Rb[ANR];
#pragma unroll
        for (int k = 0; k < M; k++) asmb[k] = aspb[k] = (T)0;
#pragma unroll
        for (int r = 0; r < ANR; r++) Rb[r] = (T)0;
        if (a.tw > 0) {
            AD::template rpt2_adj<IXY>(P, R, amf, bmmb, bpmb, asmb, Rb);
            AD::template rpt2_adj<IXY>(P, R, apf, bmpb, bppb, aspb, Rb);
        }
        T cqb[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            cqb[k] = (T)0.5 * fab[k] + (fold ? asmb[k] - aspb[k] : (T)0);
            amb[k] += asmb[k];
            apb[k] += aspb[k];
        }
        // reverse of the correction flux and of the limiter
        T Wb[MW * M], sb[MW];
#pragma unroll
        for (int f = 0; f < MW * M; f++) Wb[f] = (T)0;
#pragma unroll
        for (int p = 0; p < MW; p++) sb[p] = (T)0;
        if (a.order == 2) {
#pragma unroll
            for (int p = 0; p < MW; p++) {
                const T sa = tabs(s[p]);
                const T coef = sa * ((T)1 - sa * dtave);
                const T dcoef = (s[p] > (T)0 ? (T)1 : (s[p] < (T)0 ? (T)-1 : (T)0)) *
                                ((T)1 - (T)2 * sa * dtave);
                T wlb[M];  // adjoint of the limited wave
                T proj = (T)0;
#pragma unroll
                for (int k = 0; k < M; k++) {
                    wlb[k] = coef * cqb[k];
                    proj += phi[p] * W[p * M + k] * cqb[k];
                }
                sb[p] += dcoef * proj;
                if (upd[p] == 0) {
#pragma unroll
                    for (int k = 0; k < M; k++) Wb[p * M + k] += wlb[k];
                    continue;
                }
                const int lim = (a.mthlim >> (8 * p)) & 0xff;
                T phib = (T)0;
#pragma unroll
                for (int k = 0; k < M; k++) {
                    Wb[p * M + k] += phi[p] * wlb[k];
                    phib += W[p * M + k] * wlb[k];
                }
                const T thb = philim_deriv<T>(lim, theta[p]) * phib;
                const T dotb = thb / wn2v[p];
                const T wn2b = -thb * theta[p] / wn2v[p];
                const int nb = upd[p] < 0 ? ie - STEP : ie + STEP;
                // the neighbour edge's slot written only by this edge
                const int slot = upd[p] < 0 ? AT::GWR : AT::GWL;
#pragma unroll
                for (int k = 0; k < M; k++) {
                    const T wn = EA[(AT::FW + p * M + k) * TL::NE1 + nb];
                    Wb[p * M + k] += dotb * wn + (T)2 * wn2b * W[p * M + k];
                    GB[(slot + p * M + k) * AT::NE1 + nb] = dotb * W[p * M + k];
                }
            }
        }
#pragma unroll
        for (int f = 0; f < MW * M; f++) GB[(AT::GW + f) * AT::NE1 + ie] = Wb[f];
#pragma unroll
        for (int p = 0; p < MW; p++) GB[(AT::GS + p) * AT::NE1 + ie] = sb[p];
#pragma unroll
        for (int k = 0; k < M; k++) {
            GB[(AT::GAM + k) * AT::NE1 + ie] = amb[k];
            GB[(AT::GAP + k) * AT::NE1 + ie] = apb[k];
        }
#pragma unroll
        for (int r = 0; r < NR; r++) GB[(AT::GR + r) * AT::NE1 + ie] = Rb[r];
    }
    __syncthreads();

    // B1: reverse of the Riemann problem and of the per-cell aux values;
    // the two cells' adjoints go to the edge's first 2M EA slots
    for (int it = threadIdx.x; it < NA1 * NS; it += NT) {
        int ea, sl;
        SI::split1(it, ea, sl);
        const int cl = (IXY == 1) ? (sl + 1) * TL::QW + ea : ea * TL::QW + sl + 1;
        const int cr = cl + ((IXY == 1) ? 1 : TL::QW);
        T ql[M], qr[M], al[ANA], ar[ANA];
#pragma unroll
        for (int k = 0; k < M; k++) {
            ql[k] = QS[k * TL::QN + cl];
            qr[k] = QS[k * TL::QN + cr];
        }
#pragma unroll
        for (int f = 0; f < NA; f++) {
            al[f] = CA[f * TL::QN + cl];
            ar[f] = CA[f * TL::QN + cr];
        }
        T Wb[MW * M], sb[MW], amb[M], apb[M], Rb[ANR];
#pragma unroll
        for (int f = 0; f < MW * M; f++)
            Wb[f] = GB[(AT::GW + f) * AT::NE1 + it] + GB[(AT::GWL + f) * AT::NE1 + it] +
                    GB[(AT::GWR + f) * AT::NE1 + it];
#pragma unroll
        for (int p = 0; p < MW; p++) sb[p] = GB[(AT::GS + p) * AT::NE1 + it];
#pragma unroll
        for (int k = 0; k < M; k++) {
            amb[k] = GB[(AT::GAM + k) * AT::NE1 + it];
            apb[k] = GB[(AT::GAP + k) * AT::NE1 + it];
        }
#pragma unroll
        for (int r = 0; r < ANR; r++) Rb[r] = r < NR ? GB[(AT::GR + r) * AT::NE1 + it] : (T)0;
        T qlb[M], qrb[M], alb[ANA], arb[ANA];
#pragma unroll
        for (int k = 0; k < M; k++) qlb[k] = qrb[k] = (T)0;
#pragma unroll
        for (int f = 0; f < ANA; f++) alb[f] = arb[f] = (T)0;
        AD::template rpn2_adj<IXY>(P, ql, qr, al, ar, Wb, sb, amb, apb, Rb, qlb, qrb, alb, arb);
        AD::cell_aux_adj(P, ql, al, alb, qlb);
        AD::cell_aux_adj(P, qr, ar, arb, qrb);
#pragma unroll
        for (int k = 0; k < M; k++) {
            EA[k * TL::NE1 + it] = qlb[k];
            EA[(M + k) * TL::NE1 + it] = qrb[k];
        }
    }
    __syncthreads();

    // B0: per cell of the sweep region, add the adjoints of its two edges
    // (the edge on its low side first)
    constexpr int CW = (IXY == 1) ? TX + 4 : TX + 2, CH = (IXY == 1) ? TY + 2 : TY + 4;
    for (int it = threadIdx.x; it < CW * CH; it += NT) {
        const int cx = ((IXY == 1) ? 0 : 1) + it % CW, cy = ((IXY == 1) ? 1 : 0) + it / CW;
        const int along = (IXY == 1) ? cx : cy, sl = (IXY == 1) ? cy - 1 : cx - 1;
        const int c = cy * TL::QW + cx;
#pragma unroll
        for (int k = 0; k < M; k++) {
            T v = LA[k * TL::QN + c];
            if (along - 1 >= 0) v += EA[(M + k) * TL::NE1 + SI::item1(along - 1, sl)];  // right cell of edge along-1
            if (along < NA1) v += EA[k * TL::NE1 + SI::item1(along, sl)];               // left cell of edge along
            LA[k * TL::QN + c] = v;
        }
    }
    __syncthreads();
}

template <template <typename> class RPT, typename T, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, 1)
    adjoint_kernel(const StepArgs a, const typename RPT<T>::Params P,
                   const double *__restrict__ q, const double *__restrict__ lam_new,
                   double *lam_old, double dtdx_d, double dtdy_d) {
    using RP = RPT<T>;
    using AD = typename AdjOf<RPT>::template type<T>;
    using TL = Tile<RP, TX, TY>;
    using AT = AdjTile<RP, AD, TX, TY>;
    constexpr int M = RP::M;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *QS = reinterpret_cast<T *>(smem_raw);
    T *CA = QS + M * TL::QN;
    T *EA = CA + AT::NA * TL::QN;
    T *GB = EA + AT::EAW * TL::NE1;
    T *LT = GB + AT::GBW * TL::NE1;
    T *LA = LT + M * TX * TY;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;

    load_tile<RP, T, TX, TY, NT>(a, q, i0, j0, QS);
    for (int idx = threadIdx.x; idx < M * TX * TY; idx += NT) {
        const int k = idx / (TX * TY), c = idx % (TX * TY);
        const int gi = i0 + c % TX, gj = j0 + c / TX;
        LT[idx] = (gi < a.mx && gj < a.my)
                      ? from_double<T>(lam_new[(size_t)k + (size_t)M * ((size_t)gi + (size_t)a.mx * gj)])
                      : (T)0;
    }
    for (int idx = threadIdx.x; idx < M * TL::QN; idx += NT) LA[idx] = (T)0;
    __syncthreads();
    phase_aux<RP, T, 1, TX, TY, NT>(P, QS, CA);
    __syncthreads();
    phase_aux<RP, T, 2, TX, TY, NT>(P, QS, CA);
    __syncthreads();
    adj_sweep<RP, AD, T, 1, TX, TY, NT>(a, P, QS, CA, EA, GB, LT, LA, i0, j0, (T)dtdx_d,
                                        (T)dtdy_d);
    adj_sweep<RP, AD, T, 2, TX, TY, NT>(a, P, QS, CA, EA, GB, LT, LA, i0, j0, (T)dtdy_d,
                                        (T)dtdx_d);

    // scatter the halo region through the boundary conditions
    for (int idx = threadIdx.x; idx < M * (TX + 4) * (TY + 4); idx += NT) {
        const int k = idx % M, cell = idx / M;
        const int cx = cell % (TX + 4), cy = cell / (TX + 4);
        const T v = LA[k * TL::QN + cy * TL::QW + cx];
        if (v == (T)0) continue;
        const int gi = i0 - 2 + cx, gj = j0 - 2 + cy;
        if (gi < -2 || gi > a.mx + 1 || gj < -2 || gj > a.my + 1) continue;
        bool neg = false;
        int sj = gj, si = gi;
        if (gj < 0) {
            const int b = a.bc_lo[1];
            if (b == GCLAW_BC_EXTRAP) sj = 0;
            else if (b == GCLAW_BC_PERIODIC) sj = gj + a.my;
            else { sj = -1 - gj; neg = (k == 2); }
        } else if (gj >= a.my) {
            const int b = a.bc_hi[1];
            if (b == GCLAW_BC_EXTRAP) sj = a.my - 1;
            else if (b == GCLAW_BC_PERIODIC) sj = gj - a.my;
            else { sj = 2 * a.my - 1 - gj; neg = (k == 2); }
        }
        if (gi < 0) {
            const int b = a.bc_lo[0];
            if (b == GCLAW_BC_EXTRAP) si = 0;
            else if (b == GCLAW_BC_PERIODIC) si = gi + a.mx;
            else { si = -1 - gi; neg = neg || (k == 1); }
        } else if (gi >= a.mx) {
            const int b = a.bc_hi[0];
            if (b == GCLAW_BC_EXTRAP) si = a.mx - 1;
            else if (b == GCLAW_BC_PERIODIC) si = gi - a.mx;
            else { si = 2 * a.mx - 1 - gi; neg = neg || (k == 1); }
        }
        const double d = (double)v;
        atomicAdd(lam_old + (size_t)k + (size_t)M * ((size_t)si + (size_t)a.mx * (size_t)sj),
                  neg ? -d : d);
    }
}

template <template <typename> class RPT, typename T, int TX, int TY, int NT>
static int launch_adjoint(const gclaw_solver *s, const StepArgs &a, const double *q,
                          const double *lam_new, double *lam_old, double dt, cudaStream_t st) {
    using RP = RPT<T>;
    using AD = typename AdjOf<RPT>::template type<T>;
    using AT = AdjTile<RP, AD, TX, TY>;
    constexpr size_t smem = AT::template smem_bytes<T>();
    static_assert(smem <= 227 * 1024, "adjoint tile does not fit in shared memory");
    auto kern = adjoint_kernel<RPT, T, TX, TY, NT>;
    static unsigned long long configured = 0ull;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return GCLAW_ERR_CUDA;
    if (!(configured & (1ull << dev))) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return GCLAW_ERR_CUDA;
        configured |= 1ull << dev;
    }
    const typename RP::Params P = RP::make(s->problem_data);
    dim3 grid((s->mx + TX - 1) / TX, (s->my + TY - 1) / TY);
    kern<<<grid, NT, smem, st>>>(a, P, q, lam_new, lam_old, dt / s->dx, dt / s->dy);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

}  // namespace gclaw

using namespace gclaw;

extern "C" int gclaw_adjoint_step(const gclaw_solver *s, const double *q_dev,
                                  const double *lam_new_dev, double *lam_old_dev, double dt,
                                  void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!q_dev || !lam_new_dev || !lam_old_dev || lam_new_dev == lam_old_dev || !(dt > 0.0))
        return GCLAW_ERR_ARG;
    if ((s->rp != GCLAW_RP_ACOUSTICS_2D && s->rp != GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D) || s->capa)
        return GCLAW_ERR_UNSUPPORTED;
    int m, mw;
    gclaw_rp_shape(s->rp, &m, &mw);
    cudaStream_t st = (cudaStream_t)stream;
    // identity part of d q_new / d q_old
    if (cudaMemcpyAsync(lam_old_dev, lam_new_dev, sizeof(double) * (size_t)m * s->mx * s->my,
                        cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    StepArgs a{};
    a.dx = s->dx;
    a.dy = s->dy;
    a.mx = s->mx;
    a.my = s->my;
    for (int d = 0; d < 2; d++) {
        a.bc_lo[d] = s->bc_lower[d];
        a.bc_hi[d] = s->bc_upper[d];
    }
    a.mthlim = 0;
    for (int p = 0; p < 4; p++) a.mthlim |= (s->mthlim[p] & 0xff) << (8 * p);
    a.order = s->order;
    a.tw = s->transverse_waves;
    a.ghosted = 0;
    a.ctrl_mode = 0;
    const bool f64 = s->precision == GCLAW_PREC_FP64;
    if (s->rp == GCLAW_RP_ACOUSTICS_2D)
        return f64 ? launch_adjoint<RpAcoustics, double, 16, 16, 256>(s, a, q_dev, lam_new_dev,
                                                                      lam_old_dev, dt, st)
                   : launch_adjoint<RpAcoustics, float, 16, 16, 256>(s, a, q_dev, lam_new_dev,
                                                                     lam_old_dev, dt, st);
    return f64 ? launch_adjoint<RpShallow, double, 16, 16, 256>(s, a, q_dev, lam_new_dev,
                                                                lam_old_dev, dt, st)
               : launch_adjoint<RpShallow, float, 16, 16, 256>(s, a, q_dev, lam_new_dev,
                                                               lam_old_dev, dt, st);
}
