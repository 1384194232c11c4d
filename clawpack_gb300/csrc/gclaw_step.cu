// gclaw_step.cu -- fused classic unsplit 2D step for GB300 (sm_103a) and the
// C ABI declared in include/gclaw.h.
//
// Replaces PyClaw's ClawSolver2D._apply_bcs + classic2.step2 (upstream
// pyclaw/src/pyclaw/solver.py and pyclaw/src/pyclaw/classic/step2.f90,
// flux2.f90, limiter.f90; the pyclaw submodule is empty in the mounted
// clawpack 5.14.0 tree, meson.build:64).
//
// One CTA owns a TX x TY tile of cells and runs the whole step for it:
//   L   load the tile plus a 2-cell halo into shared memory, applying the
//       boundary conditions on the fly (extrap / periodic / wall);
//   X1  normal Riemann problems on the x-edges of rows j0-1 .. j0+TY;
//   X2  wave limiting against the upwind neighbour edge, second-order
//       correction flux, transverse splitting of A^-dq and A^+dq;
//   X3  per cell, the x-sweep contributions of rows j-1, j, j+1;
//   Y1-Y3  the same for the y-sweep on columns i0-1 .. i0+TX;
//   then each cell is written once.  The Courant number is a block max of
//   |s| reduced with one 64-bit atomicMax per block and direction; the last
//   CTA to finish turns it into the CFL and, in controlled mode, applies the
//   evolve_to_time rules to the device-resident gclaw_ctrl.
//
// The per-cell accumulation follows the serial Fortran order exactly:
//   q + [row j-1] + [row j] + [row j+1] + [col i-1] + [col i] + [col i+1].
// FP32-bulk mode sums the same terms in FP32 starting from zero and adds the
// total to the FP64 state once.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "gclaw.h"
#include "gclaw_riemann.cuh"

#define GCLAW_VERSION_STR "gclaw 0.1.0 (sm_103a)"

// Tile shape (cells per CTA in x and y, threads per CTA) per solver and
// precision, chosen by measurement on GB300 (2048^2 runs): larger tiles
// recompute fewer halo edges, which matters most for the FP64 kernels
// (FP64-pipe bound); the FP64 Euler tile is smaller because its per-edge
// records (35 doubles) must fit in shared memory.  GCLAW_TILE_F32_{TX,TY,NT}
// and GCLAW_TILE_F64_{TX,TY,NT} override every solver at build time (sweeps).
namespace gclaw {

struct StepArgs {
    const double *qin[2];
    double *qout[2];
    gclaw_ctrl *ctrl;
    double dt, dx, dy;
    int mx, my;
    int ghosted;   // input is a ghost-filled qbc (mx+4, my+4); output written at +2 offset
    int ctrl_mode; // dt / parity / done from ctrl; evolve rules in the last block
    int bc_lo[2], bc_hi[2];
    int mthlim;  // limiter id of wave p in bits 8p..8p+7
    int order, tw;
};

// Value of component k of qbc(gi, gj) for gi in [-2, mx+1], gj in [-2, my+1]
// (coordinates outside are clamped; the tile's cells past the domain only
// feed edges whose results are discarded).
template <int M>
__device__ __forceinline__ double load_q(const StepArgs &a, const double *__restrict__ q, int k,
                                         int gi, int gj) {
    gi = min(max(gi, -2), a.mx + 1);
    gj = min(max(gj, -2), a.my + 1);
    if (a.ghosted)
        return __ldg(q + k + (size_t)M * ((size_t)(gi + 2) + (size_t)(a.mx + 4) * (size_t)(gj + 2)));
    bool neg = false;
    int sj = gj;
    if (gj < 0) {
        int b = a.bc_lo[1];
        if (b == GCLAW_BC_EXTRAP) sj = 0;
        else if (b == GCLAW_BC_PERIODIC) sj = gj + a.my;
        else { sj = -1 - gj; neg = (k == 2); }
    } else if (gj >= a.my) {
        int b = a.bc_hi[1];
        if (b == GCLAW_BC_EXTRAP) sj = a.my - 1;
        else if (b == GCLAW_BC_PERIODIC) sj = gj - a.my;
        else { sj = 2 * a.my - 1 - gj; neg = (k == 2); }
    }
    int si = gi;
    if (gi < 0) {
        int b = a.bc_lo[0];
        if (b == GCLAW_BC_EXTRAP) si = 0;
        else if (b == GCLAW_BC_PERIODIC) si = gi + a.mx;
        else { si = -1 - gi; neg = neg || (k == 1); }
    } else if (gi >= a.mx) {
        int b = a.bc_hi[0];
        if (b == GCLAW_BC_EXTRAP) si = a.mx - 1;
        else if (b == GCLAW_BC_PERIODIC) si = gi - a.mx;
        else { si = 2 * a.mx - 1 - gi; neg = neg || (k == 1); }
    }
    double v = __ldg(q + k + (size_t)M * ((size_t)si + (size_t)a.mx * (size_t)sj));
    return neg ? -v : v;
}

// Exact double <-> float conversions done with integer operations.  On
// GB300 the conversion instructions issue to the FP64 pipe, which is the
// scarce unit; these give the same bits as __double2float_rn and the float
// to double widening for zeros and normal numbers and fall back to the
// instructions otherwise (denormals, very small or large magnitudes,
// infinities, NaN).
__device__ __forceinline__ float d2f_rn_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);  // +-0
    const unsigned e = (hi >> 20) & 0x7ffu;
    if (e - 897u < 253u) {  // float exponent 1..253
        unsigned f = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned rem = lo & 0x1fffffffu;
        f += (rem > 0x10000000u) | ((rem == 0x10000000u) & f);  // round to nearest even
        return __uint_as_float((hi & 0x80000000u) | f);
    }
    return __double2float_rn(x);
}

__device__ __forceinline__ double f2d_bits(float x) {
    const unsigned u = __float_as_uint(x);
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);  // +-0
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u < 254u)  // normal
        return __hiloint2double(
            (int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3)),
            (int)(u << 29));
    return (double)x;
}

template <typename T>
__device__ __forceinline__ T from_double(double v);
template <>
__device__ __forceinline__ double from_double<double>(double v) { return v; }
template <>
__device__ __forceinline__ float from_double<float>(double v) { return d2f_rn_bits(v); }

// Edge indexing of one sweep.  The x-sweep's edges sit on a (TX+3) x (TY+2)
// grid (slices are rows), the y-sweep's on a (TX+2) x (TY+3) grid (slices are
// columns).  Both are stored x-fastest, so consecutive threads touch
// consecutive x positions and shared-memory accesses are conflict-free.
//   phase 1: all edges, (ea along the slice, sl)
//   phase 2: the limited edges, (e2 = ea - 1, sl)
template <int IXY, int TX, int TY>
struct SweepIdx {
    static constexpr int NA = IXY == 1 ? TX + 3 : TY + 3;  // edges along a slice
    static constexpr int NS = IXY == 1 ? TY + 2 : TX + 2;  // slices
    static constexpr int NA2 = NA - 2;                      // limited edges per slice
    static constexpr int STEP1 = IXY == 1 ? 1 : NS;         // next edge along the sweep, phase 1
    static constexpr int STEP2 = IXY == 1 ? 1 : NS;         // next edge along the sweep, phase 2
    __device__ __forceinline__ static int item1(int ea, int sl) {
        return IXY == 1 ? sl * NA + ea : ea * NS + sl;
    }
    __device__ __forceinline__ static void split1(int it, int &ea, int &sl) {
        if (IXY == 1) { ea = it % NA; sl = it / NA; }
        else { sl = it % NS; ea = it / NS; }
    }
    __device__ __forceinline__ static int item2(int e2, int sl) {
        return IXY == 1 ? sl * NA2 + e2 : e2 * NS + sl;
    }
    __device__ __forceinline__ static void split2(int it, int &e2, int &sl) {
        if (IXY == 1) { e2 = it % NA2; sl = it / NA2; }
        else { sl = it % NS; e2 = it / NS; }
    }
};

template <template <typename> class RPT, typename T>
struct TileCfg;
#define GCLAW_TILE_CFG(RPT, T, tx, ty, nt)                           \
    template <>                                                       \
    struct TileCfg<RPT, T> {                                          \
        static constexpr int TX = tx, TY = ty, NT = nt;               \
    };
#if defined(GCLAW_TILE_F64_TX)
GCLAW_TILE_CFG(RpAcoustics, double, GCLAW_TILE_F64_TX, GCLAW_TILE_F64_TY, GCLAW_TILE_F64_NT)
GCLAW_TILE_CFG(RpShallow, double, GCLAW_TILE_F64_TX, GCLAW_TILE_F64_TY, GCLAW_TILE_F64_NT)
GCLAW_TILE_CFG(RpEuler, double, GCLAW_TILE_F64_TX, GCLAW_TILE_F64_TY, GCLAW_TILE_F64_NT)
#else
GCLAW_TILE_CFG(RpAcoustics, double, 32, 16, 256)
GCLAW_TILE_CFG(RpShallow, double, 32, 16, 256)
GCLAW_TILE_CFG(RpEuler, double, 16, 16, 256)
#endif
#if defined(GCLAW_TILE_F32_TX)
GCLAW_TILE_CFG(RpAcoustics, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
GCLAW_TILE_CFG(RpShallow, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
GCLAW_TILE_CFG(RpEuler, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
#else
GCLAW_TILE_CFG(RpAcoustics, float, 32, 16, 512)
GCLAW_TILE_CFG(RpShallow, float, 32, 16, 512)
GCLAW_TILE_CFG(RpEuler, float, 24, 16, 384)
#endif
#undef GCLAW_TILE_CFG

// Cells per CTA of the kernel that runs solver rp at the given precision.
static void tile_shape(int rp, int precision, int *tx, int *ty) {
    const bool f64 = precision == GCLAW_PREC_FP64;
    switch (rp) {
    case GCLAW_RP_ACOUSTICS_2D:
        *tx = f64 ? TileCfg<RpAcoustics, double>::TX : TileCfg<RpAcoustics, float>::TX;
        *ty = f64 ? TileCfg<RpAcoustics, double>::TY : TileCfg<RpAcoustics, float>::TY;
        return;
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D:
        *tx = f64 ? TileCfg<RpShallow, double>::TX : TileCfg<RpShallow, float>::TX;
        *ty = f64 ? TileCfg<RpShallow, double>::TY : TileCfg<RpShallow, float>::TY;
        return;
    default:
        *tx = f64 ? TileCfg<RpEuler, double>::TX : TileCfg<RpEuler, float>::TX;
        *ty = f64 ? TileCfg<RpEuler, double>::TY : TileCfg<RpEuler, float>::TY;
        return;
    }
}

template <class RP, int TX, int TY>
struct Tile {
    static constexpr int M = RP::M, MW = RP::MW, NR = RP::NR, NA = RP::NA;
    // shared-memory row stride: TX+4 cells plus one pad column so that the
    // stride is odd and column-wise (y-sweep) reads hit distinct banks
    static constexpr int QW = TX + 5, QH = TY + 4, QN = QW * QH;
    static constexpr int NE1X = (TX + 3) * (TY + 2), NE1Y = (TX + 2) * (TY + 3);
    static constexpr int NE1 = NE1X > NE1Y ? NE1X : NE1Y;
    static constexpr int NE2X = (TX + 1) * (TY + 2), NE2Y = (TX + 2) * (TY + 1);
    static constexpr int NE2 = NE2X > NE2Y ? NE2X : NE2Y;
    // edge area fields: W[MW*M], s[MW], amdq[M], apdq[M], Roe state[NR]
    static constexpr int FW = 0, FS = MW * M, FAM = FS + MW, FAP = FAM + M, FR = FAP + M;
    static constexpr int EAW = FR + NR;
    // second-phase fields: fadd, B-A-, B+A-, B-A+, B+A+ (each M)
    static constexpr int GFA = 0, GMM = M, GPM = 2 * M, GMP = 3 * M, GPP = 4 * M, EBW = 5 * M;
    // the per-cell aux values of a sweep live in the second-phase area,
    // which is free while the sweep's Riemann problems are solved
    static_assert(NA * QN <= EBW * NE2, "cell aux area does not fit");
    template <typename T>
    static constexpr size_t smem_bytes() {
        return sizeof(T) * ((size_t)M * QN + (size_t)EAW * NE1 + (size_t)EBW * NE2);
    }
};

// ---- phase 0: per-cell square roots and quotients for one sweep ---------
template <class RP, typename T, int IXY, int TX, int TY, int NT>
__device__ __forceinline__ void phase_aux(const typename RP::Params &P, const T *QS, T *CA) {
    using TL = Tile<RP, TX, TY>;
    constexpr int M = RP::M, NA = RP::NA;
    if (NA == 0) return;
    // cells the sweep's edges touch: x-sweep cx 0..TX+3, cy 1..TY+2;
    // y-sweep cx 1..TX+2, cy 0..TY+3
    constexpr int W = (IXY == 1) ? TX + 4 : TX + 2, H = (IXY == 1) ? TY + 2 : TY + 4;
    constexpr int X0 = (IXY == 1) ? 0 : 1, Y0 = (IXY == 1) ? 1 : 0;
    for (int it = threadIdx.x; it < W * H; it += NT) {
        const int c = (Y0 + it / W) * TL::QW + X0 + it % W;
        T q[M], aux[NA > 0 ? NA : 1];
#pragma unroll
        for (int k = 0; k < M; k++) q[k] = QS[k * TL::QN + c];
        RP::cell_aux(P, q, aux);
#pragma unroll
        for (int f = 0; f < NA; f++) CA[f * TL::QN + c] = aux[f];
    }
}

// ---- phase 1: normal Riemann problems on every edge of the sweep ---------
template <class RP, typename T, int IXY, int TX, int TY, int NT>
__device__ __forceinline__ void phase_rpn2(const typename RP::Params &P, const T *QS, const T *CA,
                                           T *EA, int i0, int j0, int mx, int my, T &smax,
                                           bool &bad) {
    using TL = Tile<RP, TX, TY>;
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR, NA = RP::NA;
    using SI = SweepIdx<IXY, TX, TY>;
    constexpr int NA1 = SI::NA, NS = SI::NS;
    const int gbase_e = ((IXY == 1) ? i0 : j0) - 1;
    const int gbase_s = ((IXY == 1) ? j0 : i0) - 1;
    const int n = (IXY == 1) ? mx : my, nt = (IXY == 1) ? my : mx;
    for (int it = threadIdx.x; it < NA1 * NS; it += NT) {
        int ea, sl;
        SI::split1(it, ea, sl);
        // left / lower cell and the step to the right / upper cell
        const int cl = (IXY == 1) ? (sl + 1) * TL::QW + ea : ea * TL::QW + sl + 1;
        const int cr = cl + ((IXY == 1) ? 1 : TL::QW);
        T ql[M], qr[M], al[NA > 0 ? NA : 1], ar[NA > 0 ? NA : 1];
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
        T W[MW * M], s[MW], am[M], ap[M], R[NR > 0 ? NR : 1];
        bad |= RP::template rpn2<IXY>(P, ql, qr, al, ar, W, s, am, ap, R);
#pragma unroll
        for (int f = 0; f < MW * M; f++) EA[(TL::FW + f) * TL::NE1 + it] = W[f];
#pragma unroll
        for (int p = 0; p < MW; p++) EA[(TL::FS + p) * TL::NE1 + it] = s[p];
#pragma unroll
        for (int k = 0; k < M; k++) {
            EA[(TL::FAM + k) * TL::NE1 + it] = am[k];
            EA[(TL::FAP + k) * TL::NE1 + it] = ap[k];
        }
#pragma unroll
        for (int r = 0; r < NR; r++) EA[(TL::FR + r) * TL::NE1 + it] = R[r];
        const int ge = gbase_e + ea, gs = gbase_s + sl;
        if (ea >= 1 && ea <= NA1 - 2 && ge <= n && gs <= nt) {
#pragma unroll
            for (int p = 0; p < MW; p++) {
                bad |= (s[p] != s[p]);
                smax = tmax(smax, (T)fabs(s[p]));
            }
        }
    }
}

// ---- phase 2: limiter, correction flux, transverse splitting -------------
template <class RP, typename T, int IXY, int TX, int TY, int NT>
__device__ __forceinline__ void phase_limit(const typename RP::Params &P, const T *EA, T *EB,
                                            int mthlim, int order, int tw, T dtdn) {
    using TL = Tile<RP, TX, TY>;
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR;
    using SI = SweepIdx<IXY, TX, TY>;
    constexpr int NS = SI::NS, NA2 = SI::NA2, STEP = SI::STEP1;
    for (int it = threadIdx.x; it < NA2 * NS; it += NT) {
        int e2, sl;
        SI::split2(it, e2, sl);
        const int ie = SI::item1(e2 + 1, sl);
        T W[MW * M], s[MW], am[M], ap[M], cq[M];
#pragma unroll
        for (int f = 0; f < MW * M; f++) W[f] = EA[(TL::FW + f) * TL::NE1 + ie];
#pragma unroll
        for (int p = 0; p < MW; p++) s[p] = EA[(TL::FS + p) * TL::NE1 + ie];
#pragma unroll
        for (int k = 0; k < M; k++) {
            am[k] = EA[(TL::FAM + k) * TL::NE1 + ie];
            ap[k] = EA[(TL::FAP + k) * TL::NE1 + ie];
            cq[k] = (T)0;
        }
        if (order == 2) {
#pragma unroll
            for (int p = 0; p < MW; p++) {
                const int lim = (mthlim >> (8 * p)) & 0xff;
                if (lim == 0) continue;
                T wn2 = (T)0;
#pragma unroll
                for (int k = 0; k < M; k++) wn2 = wn2 + W[p * M + k] * W[p * M + k];
                if (wn2 == (T)0) continue;
                T dot = (T)0;
                if (s[p] > (T)0) {
#pragma unroll
                    for (int k = 0; k < M; k++)
                        dot = dot + EA[(TL::FW + p * M + k) * TL::NE1 + ie - STEP] * W[p * M + k];
                } else {
#pragma unroll
                    for (int k = 0; k < M; k++)
                        dot = dot + W[p * M + k] * EA[(TL::FW + p * M + k) * TL::NE1 + ie + STEP];
                }
                const T phi = philim<T>(lim, dot / wn2);
#pragma unroll
                for (int k = 0; k < M; k++) W[p * M + k] = phi * W[p * M + k];
            }
            const T dtave = (T)0.5 * (dtdn + dtdn);
#pragma unroll
            for (int k = 0; k < M; k++) {
                T c = (T)0;
#pragma unroll
                for (int p = 0; p < MW; p++) {
                    const T sa = fabs(s[p]);
                    c = c + sa * ((T)1 - sa * dtave) * W[p * M + k];
                }
                cq[k] = c;
            }
        }
#pragma unroll
        for (int k = 0; k < M; k++) EB[(TL::GFA + k) * TL::NE2 + it] = (T)0 + (T)0.5 * cq[k];
        T bmm[M], bpm[M], bmp[M], bpp[M];
        if (tw > 0) {
            if (order == 2 && tw == 2) {
#pragma unroll
                for (int k = 0; k < M; k++) {
                    am[k] = am[k] + cq[k];
                    ap[k] = ap[k] - cq[k];
                }
            }
            T R[NR > 0 ? NR : 1];
#pragma unroll
            for (int r = 0; r < NR; r++) R[r] = EA[(TL::FR + r) * TL::NE1 + ie];
            RP::template rpt2<IXY>(P, R, am, bmm, bpm);
            RP::template rpt2<IXY>(P, R, ap, bmp, bpp);
        } else {
#pragma unroll
            for (int k = 0; k < M; k++) bmm[k] = bpm[k] = bmp[k] = bpp[k] = (T)0;
        }
#pragma unroll
        for (int k = 0; k < M; k++) {
            EB[(TL::GMM + k) * TL::NE2 + it] = bmm[k];
            EB[(TL::GPM + k) * TL::NE2 + it] = bpm[k];
            EB[(TL::GMP + k) * TL::NE2 + it] = bmp[k];
            EB[(TL::GPP + k) * TL::NE2 + it] = bpp[k];
        }
    }
}

// ---- phase 3: ordered per-cell accumulation of one sweep ------------------
// acc starts at q (FP64 mode) or 0 (FP32 mode) and receives, in order, the
// slice-before term, the own-slice term and the slice-after term.
template <class RP, typename T, typename A, int IXY, int TX, int TY, int NT, int NC>
__device__ __forceinline__ void phase_accum(const T *EA, const T *EB, A (*acc)[RP::M], T dtdn,
                                            T dtdt) {
    using TL = Tile<RP, TX, TY>;
    constexpr int M = RP::M;
    using SI = SweepIdx<IXY, TX, TY>;
    constexpr int S1 = SI::STEP1, S2 = SI::STEP2;
    const T h = (T)0.5 * dtdn;
#pragma unroll
    for (int t = 0; t < NC; t++) {
        const int n = threadIdx.x + t * NT;
        if (n >= TX * TY) break;
        const int ci = n % TX, cj = n / TX;
        const int al = (IXY == 1) ? ci : cj;   // position along the sweep
        const int so = ((IXY == 1) ? cj : ci) + 1;  // own slice
        // left / right edge of the cell in the phase-1 area, and in the
        // phase-2 area for the slice before, the own slice and the slice after
        const int el = SI::item1(al + 1, so), er = el + S1;
        const int b0 = SI::item2(al, so - 1), o0 = SI::item2(al, so), a0 = SI::item2(al, so + 1);
#pragma unroll
        for (int k = 0; k < M; k++) {
            const T *BMM = EB + (TL::GMM + k) * TL::NE2, *BPM = EB + (TL::GPM + k) * TL::NE2;
            const T *BMP = EB + (TL::GMP + k) * TL::NE2, *BPP = EB + (TL::GPP + k) * TL::NE2;
            const T *FA = EB + (TL::GFA + k) * TL::NE2;
            const T g2b = ((T)0 - h * BPM[b0 + S2]) - h * BPP[b0];
            const T qo = ((T)0 - dtdn * EA[(TL::FAP + k) * TL::NE1 + el]) -
                         dtdn * EA[(TL::FAM + k) * TL::NE1 + er];
            const T fo = FA[o0 + S2] - FA[o0];
            const T g1o = ((T)0 - h * BMM[o0 + S2]) - h * BMP[o0];
            const T g2o = ((T)0 - h * BPM[o0 + S2]) - h * BPP[o0];
            const T g1a = ((T)0 - h * BMM[a0 + S2]) - h * BMP[a0];
            A v = acc[t][k];
            v = v + (A)dtdt * (A)g2b;
            v = v + (A)qo - (A)dtdn * (A)fo - (A)dtdt * ((A)g2o - (A)g1o);
            v = v - (A)dtdt * (A)g1a;
            acc[t][k] = v;
        }
    }
}

// ---- last block: CFL and the evolve_to_time rules --------------------------
__device__ void finish_step(gclaw_ctrl *c, int ctrl_mode, double dt, double dtdx, double dtdy) {
    const double sx = __longlong_as_double((long long)atomicExch(&c->smax_bits[0], 0ull));
    const double sy = __longlong_as_double((long long)atomicExch(&c->smax_bits[1], 0ull));
    const unsigned flags = atomicExch(&c->flags, 0u);
    const double cx = dtdx * sx, cy = dtdy * sy;
    const double cfl = cx > cy ? cx : cy;
    c->cfl = cfl;
    c->blocks_done = 0u;
    if (!ctrl_mode) {
        c->status = flags ? GCLAW_NONPHYSICAL : GCLAW_OK;
        return;
    }
    c->attempts += 1;
    if (flags) {
        c->status = GCLAW_NONPHYSICAL;
        c->done = 1;
        return;
    }
    const bool accept = cfl <= c->cfl_max;
    if (accept) {
        c->cflmax = fmax(cfl, c->cflmax);
        c->numsteps += 1;
        if (c->dt_variable) c->t = c->t + dt;
        else c->t = c->t_start + (double)c->numsteps * dt;
        c->parity ^= 1;
    } else if (!c->dt_variable) {
        c->status = GCLAW_CFL_FIXED_DT;
        c->done = 1;
        return;
    }
    if (c->t >= c->t_end || (c->max_accepted >= 0 && c->numsteps >= c->max_accepted)) {
        c->done = 1;
        return;
    }
    if (c->attempts >= c->max_steps) {
        c->status = GCLAW_MAX_STEPS;
        c->done = 1;
        return;
    }
    if (c->dt_variable) {
        double ndt;
        if (cfl > 0.0) {
            ndt = fmin(c->dt_max, dt * c->cfl_desired / cfl);
            c->dtmin = fmin(ndt, c->dtmin);
            c->dtmax = fmax(ndt, c->dtmax);
        } else {
            ndt = c->dt_max;
        }
        if (c->t + ndt > c->t_end && c->t_start < c->t_end) ndt = c->t_end - c->t;
        if (c->t_end - c->t - ndt < 1.0e-14 * c->t) ndt = c->t_end - c->t;
        c->dt = ndt;
    }
}

// ---- one tile, both sweeps --------------------------------------------------
// Runs the whole step for the tile at (i0, j0): load with boundary
// conditions, both sweeps, and the write of the new state.  Returns the
// tile's max |s| on x- and y-edges and whether a Riemann problem met a
// non-physical state.  dtdx and dtdy are the block's shared copies.
template <template <typename> class RPT, typename T, int TX, int TY, int NT>
__device__ __forceinline__ void step_tile(const StepArgs &a, const typename RPT<T>::Params &P,
                                          const double *__restrict__ qin,
                                          double *__restrict__ qout, double dtdx, double dtdy,
                                          unsigned char *smem_raw, T &smax_x, T &smax_y,
                                          bool &bad) {
    using RP = RPT<T>;
    using TL = Tile<RP, TX, TY>;
    using A = T;  // FP64: accumulate q itself; FP32: accumulate the increment
    constexpr int M = RP::M;
    constexpr int NC = (TX * TY + NT - 1) / NT;
    constexpr bool FP64 = sizeof(T) == 8;
    T *QS = reinterpret_cast<T *>(smem_raw);
    T *EA = QS + M * TL::QN;
    T *EB = EA + TL::EAW * TL::NE1;
    T *CA = EB;
    const T tdtdx = (T)dtdx, tdtdy = (T)dtdy;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;

    // L: tile + halo.  When the whole window lies inside the input array
    // (every tile but the boundary ones) it is read row by row with
    // coalesced loads; otherwise each value goes through the boundary
    // conditions (load_q).
    const int off = a.ghosted ? 2 : 0, nx = a.mx + 2 * off, ny = a.my + 2 * off;
    const bool inside = i0 - 2 + off >= 0 && i0 + TX + 2 + off <= nx && j0 - 2 + off >= 0 &&
                        j0 + TY + 2 + off <= ny;
    if (inside) {
        constexpr int RW = (TX + 4) * M;  // doubles per tile row
        const double *__restrict__ base =
            qin + (size_t)M * ((size_t)(i0 - 2 + off) + (size_t)nx * (size_t)(j0 - 2 + off));
        const size_t rs = (size_t)M * (size_t)nx;
        for (int idx = threadIdx.x; idx < RW * TL::QH; idx += NT) {
            const int r = idx / RW, c = idx - r * RW;
            const int cell = c / M, k = c - cell * M;
            QS[k * TL::QN + r * TL::QW + cell] = from_double<T>(__ldg(base + r * rs + c));
        }
    } else {
        for (int idx = threadIdx.x; idx < (TX + 4) * TL::QH * M; idx += NT) {
            const int k = idx % M, cell = idx / M;
            const int cx = cell % (TX + 4), cy = cell / (TX + 4);
            QS[k * TL::QN + cy * TL::QW + cx] =
                from_double<T>(load_q<M>(a, qin, k, i0 - 2 + cx, j0 - 2 + cy));
        }
    }
    __syncthreads();

    A acc[NC][M];
#pragma unroll
    for (int t = 0; t < NC; t++) {
        const int n = threadIdx.x + t * NT;
        const int ci = n % TX, cj = n / TX;
#pragma unroll
        for (int k = 0; k < M; k++)
            acc[t][k] = (FP64 && n < TX * TY) ? QS[k * TL::QN + (cj + 2) * TL::QW + ci + 2] : (A)0;
    }

    phase_aux<RP, T, 1, TX, TY, NT>(P, QS, CA);
    __syncthreads();
    phase_rpn2<RP, T, 1, TX, TY, NT>(P, QS, CA, EA, i0, j0, a.mx, a.my, smax_x, bad);
    __syncthreads();
    phase_limit<RP, T, 1, TX, TY, NT>(P, EA, EB, a.mthlim, a.order, a.tw, tdtdx);
    __syncthreads();
    phase_accum<RP, T, A, 1, TX, TY, NT, NC>(EA, EB, acc, tdtdx, tdtdy);
    __syncthreads();
    phase_aux<RP, T, 2, TX, TY, NT>(P, QS, CA);
    __syncthreads();
    phase_rpn2<RP, T, 2, TX, TY, NT>(P, QS, CA, EA, i0, j0, a.mx, a.my, smax_y, bad);
    __syncthreads();
    phase_limit<RP, T, 2, TX, TY, NT>(P, EA, EB, a.mthlim, a.order, a.tw, tdtdy);
    __syncthreads();
    phase_accum<RP, T, A, 2, TX, TY, NT, NC>(EA, EB, acc, tdtdy, tdtdx);

    const int onx = a.ghosted ? a.mx + 4 : a.mx, ooff = a.ghosted ? 2 : 0;
#pragma unroll
    for (int t = 0; t < NC; t++) {
        const int n = threadIdx.x + t * NT;
        if (n >= TX * TY) break;
        const int gi = i0 + n % TX, gj = j0 + n / TX;
        if (gi < a.mx && gj < a.my) {
            const size_t o = (size_t)M * ((size_t)(gi + ooff) + (size_t)onx * (size_t)(gj + ooff));
#pragma unroll
            for (int k = 0; k < M; k++)
                qout[o + k] = FP64 ? (double)acc[t][k] : __ldg(qin + o + k) + f2d_bits((float)acc[t][k]);
        }
    }
}

// Block-wide max of two values of type T (result valid in thread 0) and OR
// of a flag (valid in every thread).
template <typename T, int NT>
__device__ __forceinline__ int block_reduce(T &x, T &y, bool flag, T (*red)[NT / 32]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        x = tmax(x, __shfl_xor_sync(0xffffffffu, x, off));
        y = tmax(y, __shfl_xor_sync(0xffffffffu, y, off));
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = x;
        red[1][threadIdx.x >> 5] = y;
    }
    const int any = __syncthreads_or(flag ? 1 : 0);
    if (threadIdx.x == 0) {
        for (int w = 1; w < NT / 32; w++) {
            x = tmax(x, red[0][w]);
            y = tmax(y, red[1][w]);
        }
    }
    return any;
}

template <template <typename> class RPT, typename T, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, NT <= 512 ? 2 : 1) step_kernel(const StepArgs a,
                                                  const typename RPT<T>::Params P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double s_dt, s_dtdx, s_dtdy;
    __shared__ int s_par, s_skip;
    __shared__ T s_red[2][NT / 32];

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
        s_dtdx = dt / a.dx;
        s_dtdy = dt / a.dy;
    }
    __syncthreads();
    if (s_skip) return;
    const double dt = s_dt, dtdx = s_dtdx, dtdy = s_dtdy;
    const double *__restrict__ qin = s_par ? a.qin[1] : a.qin[0];
    double *__restrict__ qout = s_par ? a.qout[1] : a.qout[0];

    T smax_x = (T)0, smax_y = (T)0;
    bool bad = false;
    step_tile<RPT, T, TX, TY, NT>(a, P, qin, qout, dtdx, dtdy, smem_raw, smax_x, smax_y, bad);

    const int anybad = block_reduce<T, NT>(smax_x, smax_y, bad, s_red);
    if (threadIdx.x == 0) {
        gclaw_ctrl *c = a.ctrl;
        atomicMax(&c->smax_bits[0], (unsigned long long)__double_as_longlong((double)smax_x));
        atomicMax(&c->smax_bits[1], (unsigned long long)__double_as_longlong((double)smax_y));
        if (anybad) atomicOr(&c->flags, 1u);
        __threadfence();
        const unsigned nblocks = gridDim.x * gridDim.y;
        const unsigned prev = atomicAdd(&c->blocks_done, 1u);
        if (prev == nblocks - 1) {
            __threadfence();
            finish_step(c, a.ctrl_mode, dt, dtdx, dtdy);
        }
    }
}

__global__ void ctrl_init_kernel(gclaw_ctrl *c, double t, double dt, double t_end, double cfl_max,
                                 double cfl_desired, double dt_max, int max_steps, int max_accepted,
                                 int dt_variable) {
    if (t + dt > t_end && t < t_end) dt = t_end - t;
    if (t_end - t - dt < 1.0e-14 * t) dt = t_end - t;
    c->t = t;
    c->dt = dt;
    c->t_start = t;
    c->t_end = t_end;
    c->cfl_max = cfl_max;
    c->cfl_desired = cfl_desired;
    c->dt_max = dt_max;
    c->cfl = 0.0;
    c->cflmax = 0.0;
    c->dtmin = dt;
    c->dtmax = dt;
    c->smax_bits[0] = 0ull;
    c->smax_bits[1] = 0ull;
    c->parity = 0;
    c->numsteps = 0;
    c->attempts = 0;
    c->max_steps = max_steps;
    c->max_accepted = max_accepted;
    c->dt_variable = dt_variable;
    c->done = (t >= t_end) ? 1 : 0;
    c->status = GCLAW_OK;
    c->blocks_done = 0u;
    c->flags = 0u;
}

// ---- launch plumbing --------------------------------------------------------
template <template <typename> class RPT, typename T, int TX, int TY, int NT>
static int launch_tile(const gclaw_solver *s, const StepArgs &a, cudaStream_t st, int nlaunch) {
    using RP = RPT<T>;
    using TL = Tile<RP, TX, TY>;
    constexpr size_t smem = TL::template smem_bytes<T>();
    auto kern = step_kernel<RPT, T, TX, TY, NT>;
    static int configured_mask = 0;  // one bit per device ordinal < 32
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GCLAW_ERR_CUDA;
    if (dev >= 32 || !(configured_mask & (1 << dev))) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return GCLAW_ERR_CUDA;
        if (dev < 32) configured_mask |= (1 << dev);
    }
    const typename RP::Params P = RP::make(s->problem_data);
    dim3 grid((s->mx + TX - 1) / TX, (s->my + TY - 1) / TY);
    for (int l = 0; l < nlaunch; l++) kern<<<grid, NT, smem, st>>>(a, P);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

template <template <typename> class RPT, typename T>
static int launch_cfg(const gclaw_solver *s, const StepArgs &a, cudaStream_t st, int nlaunch) {
    using C = TileCfg<RPT, T>;
    return launch_tile<RPT, T, C::TX, C::TY, C::NT>(s, a, st, nlaunch);
}

static int dispatch(const gclaw_solver *s, const StepArgs &a, cudaStream_t st, int nlaunch) {
    const bool f64 = s->precision == GCLAW_PREC_FP64;
    switch (s->rp) {
    case GCLAW_RP_ACOUSTICS_2D:
        return f64 ? launch_cfg<RpAcoustics, double>(s, a, st, nlaunch)
                   : launch_cfg<RpAcoustics, float>(s, a, st, nlaunch);
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D:
        return f64 ? launch_cfg<RpShallow, double>(s, a, st, nlaunch)
                   : launch_cfg<RpShallow, float>(s, a, st, nlaunch);
    case GCLAW_RP_EULER_4WAVE_2D:
        return f64 ? launch_cfg<RpEuler, double>(s, a, st, nlaunch)
                   : launch_cfg<RpEuler, float>(s, a, st, nlaunch);
    default: return GCLAW_ERR_ARG;
    }
}

static void fill_args(const gclaw_solver *s, StepArgs &a) {
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
}

}  // namespace gclaw

using namespace gclaw;

extern "C" {

const char *gclaw_version(void) { return GCLAW_VERSION_STR; }

const char *gclaw_strerror(int st) {
    switch (st) {
    case GCLAW_OK: return "ok";
    case GCLAW_ERR_ARG: return "invalid argument";
    case GCLAW_ERR_CUDA: return "CUDA error";
    case GCLAW_ERR_UNSUPPORTED: return "unsupported option";
    case GCLAW_ERR_WORKSPACE: return "workspace too small";
    case GCLAW_ERR_TOO_LARGE:
        return "grid needs more thread blocks than the no-allocation scratch holds "
               "(GCLAW_NOALLOC_MAX_BLOCKS)";
    case GCLAW_NONPHYSICAL: return "non-physical state (NaN wave speed or negative sound speed squared)";
    case GCLAW_CFL_FIXED_DT: return "CFL too large with fixed dt";
    case GCLAW_MAX_STEPS: return "maximum number of time steps taken";
    default: return "unknown status";
    }
}

int gclaw_rp_shape(int rp, int *num_eqn, int *num_waves) {
    switch (rp) {
    case GCLAW_RP_ACOUSTICS_2D: *num_eqn = 3; *num_waves = 2; return GCLAW_OK;
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D: *num_eqn = 3; *num_waves = 3; return GCLAW_OK;
    case GCLAW_RP_EULER_4WAVE_2D: *num_eqn = 4; *num_waves = 4; return GCLAW_OK;
    default: return GCLAW_ERR_ARG;
    }
}

int gclaw_check(const gclaw_solver *s) {
    int m, mw;
    if (!s || gclaw_rp_shape(s->rp, &m, &mw)) return GCLAW_ERR_ARG;
    if (s->mx < 2 || s->my < 2 || !(s->dx > 0.0) || !(s->dy > 0.0)) return GCLAW_ERR_ARG;
    if ((long long)s->mx * (long long)s->my * m > (1ll << 40)) return GCLAW_ERR_ARG;
    for (int d = 0; d < 2; d++) {
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
    if (s->order < 1 || s->order > 2 || s->transverse_waves < 0 || s->transverse_waves > 2)
        return GCLAW_ERR_ARG;
    if (s->precision != GCLAW_PREC_FP64 && s->precision != GCLAW_PREC_FP32_BULK)
        return GCLAW_ERR_ARG;
    const double *pd = s->problem_data;
    switch (s->rp) {
    case GCLAW_RP_ACOUSTICS_2D:
        if (!(pd[2] > 0.0) || !(pd[3] > 0.0)) return GCLAW_ERR_ARG;
        break;
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D:
        if (!(pd[0] > 0.0)) return GCLAW_ERR_ARG;
        break;
    default:
        if (!(pd[0] > 1.0)) return GCLAW_ERR_ARG;
        break;
    }
    return GCLAW_OK;
}

int gclaw_ctrl_init(gclaw_ctrl *ctrl_dev, double t, double dt, double t_end, double cfl_max,
                    double cfl_desired, double dt_max, int max_steps, int max_accepted,
                    int dt_variable, void *stream) {
    if (!ctrl_dev || !(dt > 0.0) || max_steps < 1) return GCLAW_ERR_ARG;
    ctrl_init_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(ctrl_dev, t, dt, t_end, cfl_max, cfl_desired,
                                                        dt_max, max_steps, max_accepted,
                                                        dt_variable ? 1 : 0);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

int gclaw_step2(const gclaw_solver *s, const double *qold_dev, double *qnew_dev, double dt,
                gclaw_ctrl *ws_dev, double *cfl_out, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!qold_dev || !qnew_dev || !ws_dev || !cfl_out || !(dt > 0.0)) return GCLAW_ERR_ARG;
    StepArgs a{};
    fill_args(s, a);
    a.qin[0] = a.qin[1] = qold_dev;
    a.qout[0] = a.qout[1] = qnew_dev;
    a.ctrl = ws_dev;
    a.dt = dt;
    a.ghosted = 1;
    a.ctrl_mode = 0;
    cudaStream_t st = (cudaStream_t)stream;
    rc = dispatch(s, a, st, 1);
    if (rc) return rc;
    double out[2];
    int status = 0;
    if (cudaMemcpyAsync(out, &ws_dev->cfl, sizeof(double), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(&status, &ws_dev->status, sizeof(int), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    *cfl_out = out[0];
    return status;
}

int gclaw_step(const gclaw_solver *s, const double *q_dev, double *qnew_dev, double dt,
               gclaw_ctrl *ws_dev, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!q_dev || !qnew_dev || !ws_dev || !(dt > 0.0)) return GCLAW_ERR_ARG;
    StepArgs a{};
    fill_args(s, a);
    a.qin[0] = a.qin[1] = q_dev;
    a.qout[0] = a.qout[1] = qnew_dev;
    a.ctrl = ws_dev;
    a.dt = dt;
    a.ghosted = 0;
    a.ctrl_mode = 0;
    return dispatch(s, a, (cudaStream_t)stream, 1);
}

int gclaw_advance(const gclaw_solver *s, double *q0_dev, double *q1_dev, gclaw_ctrl *ctrl_dev,
                  int nlaunch, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!q0_dev || !q1_dev || !ctrl_dev || nlaunch < 0) return GCLAW_ERR_ARG;
    StepArgs a{};
    fill_args(s, a);
    a.qin[0] = q0_dev;
    a.qin[1] = q1_dev;
    a.qout[0] = q1_dev;
    a.qout[1] = q0_dev;
    a.ctrl = ctrl_dev;
    a.dt = 0.0;
    a.ghosted = 0;
    a.ctrl_mode = 1;
    return dispatch(s, a, (cudaStream_t)stream, nlaunch);
}

size_t gclaw_step_workspace_bytes(const gclaw_solver *s) {
    int m, mw;
    if (!s || gclaw_rp_shape(s->rp, &m, &mw)) return 0;
    const size_t qb = sizeof(double) * (size_t)m * (size_t)s->mx * (size_t)s->my;
    const size_t qpad = (qb + 255) & ~(size_t)255;
    return 256 + 2 * qpad;
}

int gclaw_step_host(const gclaw_solver *s, const double *q_host, double *qnew_host, double dt,
                    void *ws_dev, size_t ws_bytes, double *cfl_out, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!q_host || !qnew_host || !ws_dev || !cfl_out || !(dt > 0.0)) return GCLAW_ERR_ARG;
    if (ws_bytes < gclaw_step_workspace_bytes(s)) return GCLAW_ERR_WORKSPACE;
    if (((uintptr_t)ws_dev & 255u) != 0) return GCLAW_ERR_ARG;
    int m, mw;
    gclaw_rp_shape(s->rp, &m, &mw);
    const size_t qb = sizeof(double) * (size_t)m * (size_t)s->mx * (size_t)s->my;
    const size_t qpad = (qb + 255) & ~(size_t)255;
    gclaw_ctrl *ws = (gclaw_ctrl *)ws_dev;
    double *d_q = (double *)((char *)ws_dev + 256);
    double *d_new = (double *)((char *)ws_dev + 256 + qpad);
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(d_q, q_host, qb, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    rc = gclaw_step(s, d_q, d_new, dt, ws, stream);
    if (rc) return rc;
    double cfl = 0.0;
    int status = 0;
    if (cudaMemcpyAsync(qnew_host, d_new, qb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&cfl, &ws->cfl, sizeof(double), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(&status, &ws->status, sizeof(int), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    *cfl_out = cfl;
    return status;
}

size_t gclaw_evolve_workspace_bytes(const gclaw_solver *s) {
    int m, mw;
    if (!s || gclaw_rp_shape(s->rp, &m, &mw)) return 0;
    const size_t qb = sizeof(double) * (size_t)m * (size_t)s->mx * (size_t)s->my;
    const size_t qpad = (qb + 255) & ~(size_t)255;
    return 256 + 2 * qpad;
}

int gclaw_evolve_host(const gclaw_solver *s, const double *q_host, double *q_out_host, double t,
                      double dt, double t_end, int max_accepted, double cfl_max,
                      double cfl_desired, double dt_max, int max_steps, void *ws_dev,
                      size_t ws_bytes, int batch, gclaw_ctrl *ctrl_out, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!q_host || !q_out_host || !ws_dev || !ctrl_out) return GCLAW_ERR_ARG;
    if (ws_bytes < gclaw_evolve_workspace_bytes(s)) return GCLAW_ERR_WORKSPACE;
    if (((uintptr_t)ws_dev & 255u) != 0) return GCLAW_ERR_ARG;
    if (batch <= 0) batch = 32;
    int m, mw;
    gclaw_rp_shape(s->rp, &m, &mw);
    const size_t qb = sizeof(double) * (size_t)m * (size_t)s->mx * (size_t)s->my;
    const size_t qpad = (qb + 255) & ~(size_t)255;
    gclaw_ctrl *ctrl = (gclaw_ctrl *)ws_dev;
    double *q0 = (double *)((char *)ws_dev + 256);
    double *q1 = (double *)((char *)ws_dev + 256 + qpad);
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(q0, q_host, qb, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    rc = gclaw_ctrl_init(ctrl, t, dt, t_end, cfl_max, cfl_desired, dt_max, max_steps, max_accepted,
                         1, stream);
    if (rc) return rc;
    for (;;) {
        rc = gclaw_advance(s, q0, q1, ctrl, batch, stream);
        if (rc) return rc;
        if (cudaMemcpyAsync(ctrl_out, ctrl, sizeof(gclaw_ctrl), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return GCLAW_ERR_CUDA;
        if (ctrl_out->done) break;
    }
    const double *qacc = ctrl_out->parity ? q1 : q0;
    if (cudaMemcpyAsync(q_out_host, qacc, qb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    return ctrl_out->status;
}

}  // extern "C"

// ===========================================================================
// gclaw_step2_noalloc: the classic2.step2 drop-in without a caller workspace.
//
// gclaw_step2 borrows a gclaw_ctrl from the caller as the scratch of its
// Courant-number reduction.  Some callers have no way to provide one: a
// Fortran or C host program that reaches the step through f2py or ctypes
// holding only the device arrays of the state it was handed, a process
// whose device memory is owned by another framework's caching allocator
// and must not grow behind its back, or code that has to stay
// allocation-free after start-up.  This variant keeps its scratch in
// g_noalloc_scratch, a file-scope __device__ array that every GPU loading
// the library holds until the process exits:
//   256-byte header (block counter, non-physical flag, CFL, status) +
//   one 16-byte slot per thread block (max |s| on its x- and y-edges),
//   GCLAW_NOALLOC_MAX_BLOCKS slots: 2 MiB + 256 B in total.
// Each thread block writes its slot; the last block to finish reduces all
// slots.  The caller passes the input and output states only.
// ===========================================================================
namespace gclaw {

constexpr size_t NOALLOC_HEADER_BYTES = 256;
constexpr size_t NOALLOC_SCRATCH_BYTES =
    NOALLOC_HEADER_BYTES + 16 * (size_t)GCLAW_NOALLOC_MAX_BLOCKS;

struct NoallocHeader {
    unsigned int blocks_done;  // last-block counter, zero between calls
    unsigned int flags;        // non-physical flag of this call
    int status;                // GCLAW_OK or GCLAW_NONPHYSICAL
    int pad;
    double cfl;                // Courant number of this call
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

template <template <typename> class RPT, typename T, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, NT <= 512 ? 2 : 1)
    step_kernel_noalloc(const StepArgs a, const typename RPT<T>::Params P,
                        unsigned char *__restrict__ scratch) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double s_dtdx, s_dtdy;
    __shared__ T s_red[2][NT / 32];
    __shared__ double s_fin[2][NT / 32];
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        s_dtdx = a.dt / a.dx;
        s_dtdy = a.dt / a.dy;
    }
    __syncthreads();
    const double dtdx = s_dtdx, dtdy = s_dtdy;

    T smax_x = (T)0, smax_y = (T)0;
    bool bad = false;
    step_tile<RPT, T, TX, TY, NT>(a, P, a.qin[0], a.qout[0], dtdx, dtdy, smem_raw, smax_x,
                                  smax_y, bad);
    const int anybad = block_reduce<T, NT>(smax_x, smax_y, bad, s_red);

    NoallocHeader *hdr = reinterpret_cast<NoallocHeader *>(scratch);
    double2 *slots = reinterpret_cast<double2 *>(scratch + NOALLOC_HEADER_BYTES);
    const unsigned nblocks = gridDim.x * gridDim.y;
    if (threadIdx.x == 0) {
        slots[blockIdx.y * gridDim.x + blockIdx.x] = make_double2((double)smax_x, (double)smax_y);
        if (anybad) atomicOr(&hdr->flags, 1u);
        __threadfence();
        s_last = (atomicAdd(&hdr->blocks_done, 1u) == nblocks - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double mx = 0.0, my = 0.0;
    for (unsigned b = threadIdx.x; b < nblocks; b += NT) {
        const double2 v = __ldcg(&slots[b]);
        mx = fmax(mx, v.x);
        my = fmax(my, v.y);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        my = fmax(my, __shfl_xor_sync(0xffffffffu, my, off));
    }
    if ((threadIdx.x & 31) == 0) {
        s_fin[0][threadIdx.x >> 5] = mx;
        s_fin[1][threadIdx.x >> 5] = my;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < NT / 32; w++) {
            mx = fmax(mx, s_fin[0][w]);
            my = fmax(my, s_fin[1][w]);
        }
        const double cx = dtdx * mx, cy = dtdy * my;
        hdr->cfl = cx > cy ? cx : cy;
        hdr->status = atomicExch(&hdr->flags, 0u) ? GCLAW_NONPHYSICAL : GCLAW_OK;
        hdr->blocks_done = 0u;
    }
}

// Device address of g_noalloc_scratch, looked up once per device.
static void *g_noalloc_ptr[64];

template <template <typename> class RPT, typename T, int TX, int TY, int NT>
static int launch_noalloc(const gclaw_solver *s, const StepArgs &a, cudaStream_t st,
                          unsigned char *scratch) {
    using RP = RPT<T>;
    using TL = Tile<RP, TX, TY>;
    constexpr size_t smem = TL::template smem_bytes<T>();
    auto kern = step_kernel_noalloc<RPT, T, TX, TY, NT>;
    const long long nblocks =
        (long long)((s->mx + TX - 1) / TX) * (long long)((s->my + TY - 1) / TY);
    if (nblocks > GCLAW_NOALLOC_MAX_BLOCKS) return GCLAW_ERR_TOO_LARGE;
    static unsigned long long configured = 0ull;  // one bit per device ordinal
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return GCLAW_ERR_CUDA;
    if (!(configured & (1ull << dev))) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return GCLAW_ERR_CUDA;
        configured |= 1ull << dev;
    }
    if (cudaMemsetAsync(scratch, 0, NOALLOC_HEADER_BYTES, st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    const typename RP::Params P = RP::make(s->problem_data);
    dim3 grid((s->mx + TX - 1) / TX, (s->my + TY - 1) / TY);
    kern<<<grid, NT, smem, st>>>(a, P, scratch);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

}  // namespace gclaw

extern "C" int gclaw_step2_noalloc(const gclaw_solver *s, const double *qold_dev,
                                   double *qnew_dev, double dt, double *cfl_out, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    // size first: a grid beyond the scratch is refused whatever the pointers
    const bool f64 = s->precision == GCLAW_PREC_FP64;
    int tx, ty;
    tile_shape(s->rp, s->precision, &tx, &ty);
    const long long tiles_x = (s->mx + tx - 1) / tx, tiles_y = (s->my + ty - 1) / ty;
    if (tiles_x * tiles_y > GCLAW_NOALLOC_MAX_BLOCKS) return GCLAW_ERR_TOO_LARGE;
    if (!qold_dev || !qnew_dev || !cfl_out || !(dt > 0.0)) return GCLAW_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return GCLAW_ERR_CUDA;
    if (!g_noalloc_ptr[dev]) {
        // first call on this device: the device address of the file-scope
        // scratch (the host-side name is only a stand-in for it)
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
            return GCLAW_ERR_CUDA;
        g_noalloc_ptr[dev] = p;
    }
    unsigned char *scratch = (unsigned char *)g_noalloc_ptr[dev];
    StepArgs a{};
    fill_args(s, a);
    a.qin[0] = a.qin[1] = qold_dev;
    a.qout[0] = a.qout[1] = qnew_dev;
    a.ctrl = nullptr;
    a.dt = dt;
    a.ghosted = 1;
    a.ctrl_mode = 0;
    cudaStream_t st = (cudaStream_t)stream;
#define GCLAW_LAUNCH_NA(RPT)                                                             \
    (f64 ? launch_noalloc<RPT, double, TileCfg<RPT, double>::TX, TileCfg<RPT, double>::TY, \
                          TileCfg<RPT, double>::NT>(s, a, st, scratch)                    \
         : launch_noalloc<RPT, float, TileCfg<RPT, float>::TX, TileCfg<RPT, float>::TY,   \
                          TileCfg<RPT, float>::NT>(s, a, st, scratch))
    switch (s->rp) {
    case GCLAW_RP_ACOUSTICS_2D: rc = GCLAW_LAUNCH_NA(RpAcoustics); break;
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D: rc = GCLAW_LAUNCH_NA(RpShallow); break;
    default: rc = GCLAW_LAUNCH_NA(RpEuler); break;
    }
#undef GCLAW_LAUNCH_NA
    if (rc) return rc;
    NoallocHeader h;
    if (cudaMemcpyAsync(&h, scratch, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    *cfl_out = h.cfl;
    return h.status;
}
