// gclaw_step_impl.cuh -- device code shared by the single-problem step
// (gclaw_step.cu) and the batched step (gclaw_batch.cu): tile shapes, the
// phases of one tile of the classic unsplit step, the tile body step_tile,
// block reductions and the evolve_to_time rules applied by the last block.
// See gclaw_step.cu for the description of the phases.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gclaw.h"
#include "gclaw_riemann.cuh"

namespace gclaw {

// Division of a 32-bit index by a runtime divisor d >= 2 as a multiply-high
// and a shift (Granlund and Montgomery, PLDI 1994): with l = ceil(log2 d)
// and m = ceil(2^(31 + l) / d), which is below 2^32, floor(n / d) equals
// umulhi(n, m) >> (l - 1) for every n < 2^31.
struct Divisor {
    unsigned m;
    int s, d;
};
static Divisor make_divisor(int d) {
    int l = 0;
    while ((1ll << l) < d) l++;
    const unsigned long long m = ((1ull << (31 + l)) + (unsigned long long)d - 1) / d;
    return Divisor{(unsigned)m, l - 1, d};
}
__device__ __forceinline__ unsigned udiv(unsigned n, const Divisor &v) {
    return __umulhi(n, v.m) >> v.s;
}

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
    const double *aux;           // per-cell aux (user aux of the solver, then the capacity)
    int maux;                    // fields per cell of aux, laid out like q
    int abc_lo[2], abc_hi[2];    // its boundary conditions (walls mirror, no negation)
    int sweeps;     // 1: x-sweep only, 2: y-sweep only (dimensional splitting); else both
    int no_finish;  // last block resets the block counter but leaves the CFL
                    // reduction to the next launch (first sweep of a split step)
    int ty0, nty;   // tile rows [ty0, ty0 + nty) only (nty > 0): one band of a
                    // step launched band by band; nty = 0: the whole grid
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
    const double v = __ldg(q + k + (size_t)M * ((size_t)si + (size_t)a.mx * (size_t)sj));
    // sign flip on the integer pipes (a negation would be an FP64 instruction)
    return __longlong_as_double(__double_as_longlong(v) ^
                                (neg ? (long long)0x8000000000000000ull : 0ll));
}

// Component k of the ghost-filled aux array at (gi, gj), as load_q maps q but
// with the aux boundary conditions (a wall mirrors without negation).
__device__ __forceinline__ double load_a(const StepArgs &a, int k, int gi, int gj) {
    gi = min(max(gi, -2), a.mx + 1);
    gj = min(max(gj, -2), a.my + 1);
    const size_t NUA = (size_t)a.maux;
    if (a.ghosted)
        return __ldg(a.aux + k + NUA * ((size_t)(gi + 2) + (size_t)(a.mx + 4) * (size_t)(gj + 2)));
    int sj = gj, si = gi;
    if (gj < 0) {
        const int b = a.abc_lo[1];
        sj = b == GCLAW_BC_EXTRAP ? 0 : (b == GCLAW_BC_PERIODIC ? gj + a.my : -1 - gj);
    } else if (gj >= a.my) {
        const int b = a.abc_hi[1];
        sj = b == GCLAW_BC_EXTRAP ? a.my - 1 : (b == GCLAW_BC_PERIODIC ? gj - a.my : 2 * a.my - 1 - gj);
    }
    if (gi < 0) {
        const int b = a.abc_lo[0];
        si = b == GCLAW_BC_EXTRAP ? 0 : (b == GCLAW_BC_PERIODIC ? gi + a.mx : -1 - gi);
    } else if (gi >= a.mx) {
        const int b = a.abc_hi[0];
        si = b == GCLAW_BC_EXTRAP ? a.mx - 1 : (b == GCLAW_BC_PERIODIC ? gi - a.mx : 2 * a.mx - 1 - gi);
    }
    return __ldg(a.aux + k + NUA * ((size_t)si + (size_t)a.mx * (size_t)sj));
}

// Solvers that read a user aux array (gclaw_solver.aux), and its fields.
inline bool rp_user_aux(int rp) {
    return rp == GCLAW_RP_VC_ACOUSTICS_2D || rp == GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D;
}
inline int rp_num_aux(int rp) {
    return rp == GCLAW_RP_VC_ACOUSTICS_2D ? 2 : (rp == GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D ? 1 : 0);
}

// Solver RPT with a capacity function kappa (classic2's mcapa): the user aux
// array gains a last field, kappa, kept in aux-area plane KAP after the
// solver's own planes.  The step then takes dt / (kappa dx) per cell for the
// fluctuations, Courant numbers and transverse terms, the mean of an edge's
// two cells in the correction flux, and divides the flux differences of a
// cell by its kappa (capacity-form differencing, LeVeque 1997 sec. 5).
template <template <typename> class RPT>
struct Capa {
    template <typename T>
    struct rp : RPT<T> {
        using B = RPT<T>;
        static constexpr int NUA = B::NUA + 1, NA = B::NA + 1, KAP = B::NA;
        static constexpr bool CAPA = true;
        __device__ __forceinline__ static void cell_aux_user(const typename B::Params &P,
                                                             const T *q, T *aux) {
            if constexpr (B::NUA > 0) B::cell_aux_user(P, q, aux);
            else if constexpr (B::NA > 0) B::cell_aux(P, q, aux);
        }
    };
};

// Aux-area plane of the capacity (solvers wrapped in Capa only).
template <class RP>
__host__ __device__ constexpr int capa_plane() {
    if constexpr (RP::CAPA) return RP::KAP;
    else return 0;
}

// Exact double <-> float conversions done with integer operations.  On
// GB300 the conversion instructions issue to the FP64 pipe, which is the
// scarce unit; these give the same bits as __double2float_rn and the float
// to double widening for zeros and normal numbers and fall back to the
// instructions otherwise (denormals, very small or large magnitudes,
// infinities, NaN).
// The uncommon cases go through real calls, so that the compiler branches
// around the conversion instruction instead of executing it for every value
// and selecting.
static __device__ __noinline__ float d2f_slow(double x) { return __double2float_rn(x); }
static __device__ __noinline__ double f2d_slow(float x) { return (double)x; }

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
    return d2f_slow(x);
}

__device__ __forceinline__ double f2d_bits(float x) {
    const unsigned u = __float_as_uint(x);
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);  // +-0
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u < 254u)  // normal
        return __hiloint2double(
            (int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3)),
            (int)(u << 29));
    return f2d_slow(x);
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

// Tile shape (cells per CTA in x and y, threads per CTA) per solver and
// precision, chosen by measurement on GB300 (2048^2 runs): larger tiles
// recompute fewer halo edges, which matters most for the FP64 kernels
// (FP64-pipe bound); the FP64 Euler tile is smaller because its per-edge
// records (35 doubles) must fit in shared memory.  GCLAW_TILE_F32_{TX,TY,NT}
// and GCLAW_TILE_F64_{TX,TY,NT} override every solver at build time (sweeps).
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
GCLAW_TILE_CFG(RpVcAcoustics, double, GCLAW_TILE_F64_TX, GCLAW_TILE_F64_TY, GCLAW_TILE_F64_NT)
GCLAW_TILE_CFG(RpShallowFwave, double, GCLAW_TILE_F64_TX, GCLAW_TILE_F64_TY, GCLAW_TILE_F64_NT)
#else
GCLAW_TILE_CFG(RpShallowFwave, double, 32, 16, 256)
GCLAW_TILE_CFG(RpVcAcoustics, double, 32, 16, 256)
GCLAW_TILE_CFG(RpAcoustics, double, 32, 16, 256)
GCLAW_TILE_CFG(RpShallow, double, 32, 16, 256)
GCLAW_TILE_CFG(RpEuler, double, 16, 16, 256)
#endif
#if defined(GCLAW_TILE_F32_TX)
GCLAW_TILE_CFG(RpAcoustics, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
GCLAW_TILE_CFG(RpShallow, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
GCLAW_TILE_CFG(RpEuler, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
GCLAW_TILE_CFG(RpVcAcoustics, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
GCLAW_TILE_CFG(RpShallowFwave, float, GCLAW_TILE_F32_TX, GCLAW_TILE_F32_TY, GCLAW_TILE_F32_NT)
#else
GCLAW_TILE_CFG(RpShallowFwave, float, 32, 16, 512)
GCLAW_TILE_CFG(RpVcAcoustics, float, 32, 16, 512)
GCLAW_TILE_CFG(RpAcoustics, float, 32, 16, 512)
GCLAW_TILE_CFG(RpShallow, float, 32, 16, 512)
GCLAW_TILE_CFG(RpEuler, float, 24, 16, 384)
#endif
#undef GCLAW_TILE_CFG

// Tile of the capacity variant: the solver's tile with TY lowered (by 2)
// until the per-tile aux area, one plane larger, fits beside the rest.
template <class RP, typename T, int TX, int TY>
constexpr int capa_fit_ty();
template <template <typename> class RPT, typename T>
struct CapaTileCfg {
    static constexpr int TX = TileCfg<RPT, T>::TX, NT = TileCfg<RPT, T>::NT;
    static constexpr int TY =
        capa_fit_ty<typename Capa<RPT>::template rp<T>, T, TX, TileCfg<RPT, T>::TY>();
};

// Resident CTAs per SM the tile kernels are compiled for (the register cap):
// two, except FP64 tiles of more than 256 threads, which hold one CTA per SM
// anyway (their per-tile aux area fills the shared memory) and may then use
// up to 128 registers a thread.
template <typename T, int NT>
__host__ __device__ constexpr int tile_min_blocks() {
    return (NT <= 256 || sizeof(T) == 4) && NT <= 512 ? 2 : 1;
}

// Cells per CTA of the kernel that runs solver rp at the given precision.
static inline void tile_shape(int rp, int precision, int *tx, int *ty) {
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
    case GCLAW_RP_VC_ACOUSTICS_2D:
        *tx = f64 ? TileCfg<RpVcAcoustics, double>::TX : TileCfg<RpVcAcoustics, float>::TX;
        *ty = f64 ? TileCfg<RpVcAcoustics, double>::TY : TileCfg<RpVcAcoustics, float>::TY;
        return;
    case GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D:
        *tx = f64 ? TileCfg<RpShallowFwave, double>::TX : TileCfg<RpShallowFwave, float>::TX;
        *ty = f64 ? TileCfg<RpShallowFwave, double>::TY : TileCfg<RpShallowFwave, float>::TY;
        return;
    default:
        *tx = f64 ? TileCfg<RpEuler, double>::TX : TileCfg<RpEuler, float>::TX;
        *ty = f64 ? TileCfg<RpEuler, double>::TY : TileCfg<RpEuler, float>::TY;
        return;
    }
}

// Wave components a solver can make nonzero (the same count in both
// directions), and the compact shared-memory plane of component k of wave p
// in direction IXY: components that are zero by the eigenstructure get no
// plane.
template <class RP>
__host__ __device__ constexpr int wave_planes() {
    int n = 0;
    for (int p = 0; p < RP::MW; p++)
        for (int k = 0; k < RP::M; k++) n += RP::template wnz<1>(p, k) ? 1 : 0;
    return n;
}
template <class RP, int IXY>
__host__ __device__ constexpr int wave_plane(int p, int k) {
    int n = 0;
    for (int pp = 0; pp < RP::MW; pp++)
        for (int kk = 0; kk < RP::M; kk++) {
            if (pp == p && kk == k) return n;
            n += RP::template wnz<IXY>(pp, kk) ? 1 : 0;
        }
    return n;
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
    // edge area fields: nonzero wave components, s[MW], amdq[M], apdq[M],
    // Roe state[NR]
    static constexpr int NWP = wave_planes<RP>();
    static constexpr int FW = 0, FS = NWP, FAM = FS + MW, FAP = FAM + M, FR = FAP + M;
    static constexpr int EAW = FR + NR;
    // second-phase fields: fadd, B-A-, B+A-, B-A+, B+A+ (each M)
    static constexpr int GFA = 0, GMM = M, GPM = 2 * M, GMP = 3 * M, GPP = 4 * M, EBW = 5 * M;
    // The per-cell aux values get their own area, computed once per tile for
    // both sweeps, when that still fits the occupancy the kernel is built
    // for (one CTA per SM in FP64, two in FP32); otherwise each sweep
    // computes them into the second-phase area, which is free while the
    // sweep's Riemann problems are solved.
    template <typename T>
    __host__ __device__ static constexpr size_t base_bytes() {
        return sizeof(T) * ((size_t)M * QN + (size_t)EAW * NE1 + (size_t)EBW * NE2);
    }
    template <typename T>
    __host__ __device__ static constexpr bool aux_own() {
        return base_bytes<T>() + sizeof(T) * (size_t)NA * QN <=
               (sizeof(T) == 8 ? (size_t)230000 : (size_t)115000);
    }
    template <typename T>
    __host__ __device__ static constexpr size_t smem_bytes() {
        return base_bytes<T>() + (aux_own<T>() ? sizeof(T) * (size_t)NA * QN : 0);
    }
};

template <class RP, typename T, int TX, int TY>
constexpr int capa_fit_ty() {
    if constexpr (TY <= 2 || Tile<RP, TX, TY>::template aux_own<T>()) return TY;
    else return capa_fit_ty<RP, T, TX, TY - 2>();
}

// ---- phase 0: per-cell square roots and quotients for one sweep ---------
template <class RP, typename T, int IXY, int TX, int TY, int NT>
__device__ __forceinline__ void phase_aux(const typename RP::Params &P, const T *QS, T *CA) {
    static_assert(RP::NUA <= RP::NA, "user aux is the first planes of the aux area");
    using TL = Tile<RP, TX, TY>;
    constexpr int M = RP::M, NA = RP::NA;
    if (NA == 0) return;
    // cells the sweep's edges touch: x-sweep cx 0..TX+3, cy 1..TY+2;
    // y-sweep cx 1..TX+2, cy 0..TY+3; IXY = 0: every cell of the tile and
    // its halo, for both sweeps
    constexpr int W = (IXY == 2) ? TX + 2 : TX + 4, H = (IXY == 1) ? TY + 2 : TY + 4;
    constexpr int X0 = (IXY == 2) ? 1 : 0, Y0 = (IXY == 1) ? 1 : 0;
    for (int it = threadIdx.x; it < W * H; it += NT) {
        const int c = (Y0 + it / W) * TL::QW + X0 + it % W;
        T q[M], aux[NA > 0 ? NA : 1];
#pragma unroll
        for (int k = 0; k < M; k++) q[k] = QS[k * TL::QN + c];
        if constexpr (RP::NUA > 0) {
            // the user aux was loaded into CA with the tile; transform in place
#pragma unroll
            for (int f = 0; f < NA; f++) aux[f] = CA[f * TL::QN + c];
            RP::cell_aux_user(P, q, aux);
        } else {
            RP::cell_aux(P, q, aux);
        }
#pragma unroll
        for (int f = 0; f < NA; f++) CA[f * TL::QN + c] = aux[f];
    }
}

// ---- phase 1: normal Riemann problems on every edge of the sweep ---------
template <class RP, typename T, int IXY, int TX, int TY, int NT>
__device__ __forceinline__ void phase_rpn2(const typename RP::Params &P, const T *QS, const T *CA,
                                           T *EA, int i0, int j0, int mx, int my, T dtdn, T &smax,
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
        if constexpr (RP::TNB) {
            // aux of the cells below / above the two edge cells (transverse)
            constexpr int TS = (IXY == 1) ? TL::QW : 1;
            T bl[NA], tl[NA], br[NA], tr[NA];
#pragma unroll
            for (int f = 0; f < NA; f++) {
                bl[f] = CA[f * TL::QN + cl - TS];
                tl[f] = CA[f * TL::QN + cl + TS];
                br[f] = CA[f * TL::QN + cr - TS];
                tr[f] = CA[f * TL::QN + cr + TS];
            }
            bad |= RP::template rpn2_nb<IXY>(P, ql, qr, al, ar, bl, tl, br, tr, W, s, am, ap, R);
        } else {
            bad |= RP::template rpn2<IXY>(P, ql, qr, al, ar, W, s, am, ap, R);
        }
#pragma unroll
        for (int f = 0; f < MW * M; f++)
            if (RP::template wnz<IXY>(f / M, f % M))
                EA[(TL::FW + wave_plane<RP, IXY>(f / M, f % M)) * TL::NE1 + it] = W[f];
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
            if constexpr (RP::CAPA) {
                // Courant numbers themselves: dt / (kappa dx) of the cell
                // downwind of each wave, times |s|
                const T dl = dtdn / CA[RP::KAP * TL::QN + cl], dr = dtdn / CA[RP::KAP * TL::QN + cr];
#pragma unroll
                for (int p = 0; p < MW; p++) {
                    bad |= isnan_v(s[p]);
                    smax = max_abs(smax, gt0(s[p]) ? dr * s[p] : dl * s[p]);
                }
            } else {
#pragma unroll
                for (int p = 0; p < MW; p++) {
                    bad |= isnan_v(s[p]);
                    smax = max_abs(smax, s[p]);
                }
            }
        }
    }
}

// ---- phase 2: limiter, correction flux, transverse splitting -------------
template <class RP, typename T, int IXY, int TX, int TY, int NT>
__device__ __forceinline__ void phase_limit(const typename RP::Params &P, const T *EA, T *EB,
                                            const T *CA, int mthlim, int order, int tw, T dtdn) {
    using TL = Tile<RP, TX, TY>;
    constexpr int M = RP::M, MW = RP::MW, NR = RP::NR;
    using SI = SweepIdx<IXY, TX, TY>;
    constexpr int NS = SI::NS, NA2 = SI::NA2, STEP = SI::STEP1;
    for (int it = threadIdx.x; it < NA2 * NS; it += NT) {
        int e2, sl;
        SI::split2(it, e2, sl);
        const int ie = SI::item1(e2 + 1, sl);
        T W[MW * M], s[MW], am[M], ap[M], cq[M];
        // components that are zero by the solver's eigenstructure are neither
        // stored nor loaded; the sums below then skip exact +0 terms
#pragma unroll
        for (int f = 0; f < MW * M; f++)
            W[f] = RP::template wnz<IXY>(f / M, f % M)
                       ? EA[(TL::FW + wave_plane<RP, IXY>(f / M, f % M)) * TL::NE1 + ie]
                       : (T)0;
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
                for (int k = 0; k < M; k++)
                    if (RP::template wnz<IXY>(p, k)) wn2 = wn2 + W[p * M + k] * W[p * M + k];
                if (eq0(wn2)) continue;
                T dot = (T)0;
                if (gt0(s[p])) {
#pragma unroll
                    for (int k = 0; k < M; k++)
                        if (RP::template wnz<IXY>(p, k))
                            dot = dot + EA[(TL::FW + wave_plane<RP, IXY>(p, k)) * TL::NE1 + ie - STEP] *
                                            W[p * M + k];
                } else {
#pragma unroll
                    for (int k = 0; k < M; k++)
                        if (RP::template wnz<IXY>(p, k))
                            dot = dot + W[p * M + k] *
                                            EA[(TL::FW + wave_plane<RP, IXY>(p, k)) * TL::NE1 + ie + STEP];
                }
                // theta = dot / wn2 <= 0 gives phi = 0 for every limiter id
                // (1-4), so the quotient is only taken for dot > 0
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
            T dtave = (T)0.5 * (dtdn + dtdn);
            if constexpr (RP::CAPA) {  // the mean dt / (kappa dx) of the edge's two cells
                const int ea = e2 + 1;
                const int cl = (IXY == 1) ? (sl + 1) * TL::QW + ea : ea * TL::QW + sl + 1;
                const int cr = cl + ((IXY == 1) ? 1 : TL::QW);
                dtave = (T)0.5 * (dtdn / CA[RP::KAP * TL::QN + cl] + dtdn / CA[RP::KAP * TL::QN + cr]);
            }
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
            if constexpr (RP::TNB) {
                RP::template rpt2s<IXY, 0>(P, R, am, bmm, bpm);
                RP::template rpt2s<IXY, 1>(P, R, ap, bmp, bpp);
            } else {
                RP::template rpt2<IXY>(P, R, am, bmm, bpm);
                RP::template rpt2<IXY>(P, R, ap, bmp, bpp);
            }
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
__device__ __forceinline__ void phase_accum(const T *EA, const T *EB, const T *CA,
                                            A (*acc)[RP::M], T dtdn, T dtdt) {
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
        if constexpr (RP::CAPA) {
            // capacity form: dt / (kappa dx) of the cell each term belongs
            // to, and the flux differences over this cell's kappa
            constexpr int TS = (IXY == 1) ? TL::QW : 1;
            const int c0 = (cj + 2) * TL::QW + ci + 2;
            const T *K = CA + RP::KAP * TL::QN;
            const T ko = K[c0];
            const T dto = dtdn / ko;
            const T hb = (T)0.5 * (dtdn / K[c0 - TS]), ho = (T)0.5 * dto,
                    ha = (T)0.5 * (dtdn / K[c0 + TS]);
#pragma unroll
            for (int k = 0; k < M; k++) {
                const T *BMM = EB + (TL::GMM + k) * TL::NE2, *BPM = EB + (TL::GPM + k) * TL::NE2;
                const T *BMP = EB + (TL::GMP + k) * TL::NE2, *BPP = EB + (TL::GPP + k) * TL::NE2;
                const T *FA = EB + (TL::GFA + k) * TL::NE2;
                const T g2b = ((T)0 - hb * BPM[b0 + S2]) - hb * BPP[b0];
                const T qo = ((T)0 - dto * EA[(TL::FAP + k) * TL::NE1 + el]) -
                             dto * EA[(TL::FAM + k) * TL::NE1 + er];
                const T fo = FA[o0 + S2] - FA[o0];
                const T g1o = ((T)0 - ho * BMM[o0 + S2]) - ho * BMP[o0];
                const T g2o = ((T)0 - ho * BPM[o0 + S2]) - ho * BPP[o0];
                const T g1a = ((T)0 - ha * BMM[a0 + S2]) - ha * BMP[a0];
                A v = acc[t][k];
                v = v + (A)dtdt * (A)g2b / (A)ko;
                v = v + (A)qo - ((A)dtdn * (A)fo + (A)dtdt * ((A)g2o - (A)g1o)) / (A)ko;
                v = v - (A)dtdt * (A)g1a / (A)ko;
                acc[t][k] = v;
            }
            continue;
        }
#pragma unroll
        for (int k = 0; k < M; k++) {
            const T *BMM = EB + (TL::GMM + k) * TL::NE2, *BPM = EB + (TL::GPM + k) * TL::NE2;
            const T *BMP = EB + (TL::GMP + k) * TL::NE2, *BPP = EB + (TL::GPP + k) * TL::NE2;
            const T *FA = EB + (TL::GFA + k) * TL::NE2;
#ifndef GCLAW_STRICT
            // FP64: the same terms regrouped: the first-order and correction
            // parts share the factor dt/dn and the eight transverse parts the
            // factor (dt/dt') h, so the cell takes two multiply-adds instead of
            // the reference's term-by-term sequence (GCLAW_STRICT keeps that;
            // in FP32 the longer-lived sums cost a register spill, so FP32
            // keeps it too).
            if constexpr (sizeof(T) == 8) {
                const T s1 = (EA[(TL::FAP + k) * TL::NE1 + el] + EA[(TL::FAM + k) * TL::NE1 + er]) +
                             (FA[o0 + S2] - FA[o0]);
                const T tb = ((BPM[b0 + S2] + BPP[b0]) - (BPM[o0 + S2] + BPP[o0])) +
                             ((BMM[o0 + S2] + BMP[o0]) - (BMM[a0 + S2] + BMP[a0]));
                A v = acc[t][k];
                v = v - (A)dtdn * (A)s1;
                v = v - (A)(dtdt * h) * (A)tb;
                acc[t][k] = v;
                continue;
            }
#endif
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
static __device__ void finish_step(gclaw_ctrl *c, int ctrl_mode, double dt, double dtdx,
                                   double dtdy) {
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

// ---- tile load ---------------------------------------------------------------
// The tile at (i0, j0) plus its 2-cell halo into QS (SoA planes, row stride
// QW).  When the whole window lies inside the input array (every tile but
// the boundary ones) it is read row by row with coalesced loads; otherwise
// each value goes through the boundary conditions (load_q).
template <class RP, typename T, int TX, int TY, int NT>
__device__ __forceinline__ void load_tile(const StepArgs &a, const double *__restrict__ qin, int i0,
                                          int j0, T *QS, T *CA = nullptr) {
    using TL = Tile<RP, TX, TY>;
    constexpr int M = RP::M;
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
    if constexpr (RP::NUA > 0) {
        // user aux of the tile and its halo, into the per-cell aux area
        for (int idx = threadIdx.x; idx < (TX + 4) * TL::QH * RP::NUA; idx += NT) {
            const int k = idx % RP::NUA, cell = idx / RP::NUA;
            const int cx = cell % (TX + 4), cy = cell / (TX + 4);
            // the capacity (last user field) goes to its own plane
            const int plane = (RP::CAPA && k == RP::NUA - 1) ? capa_plane<RP>() : k;
            CA[plane * TL::QN + cy * TL::QW + cx] =
                from_double<T>(load_a(a, k, i0 - 2 + cx, j0 - 2 + cy));
        }
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
                                          int i0, int j0, unsigned char *smem_raw, T &smax_x,
                                          T &smax_y, bool &bad) {
    using RP = RPT<T>;
    using TL = Tile<RP, TX, TY>;
    using A = T;  // FP64: accumulate q itself; FP32: accumulate the increment
    constexpr int M = RP::M;
    constexpr int NC = (TX * TY + NT - 1) / NT;
    constexpr bool FP64 = sizeof(T) == 8;
    T *QS = reinterpret_cast<T *>(smem_raw);
    T *EA = QS + M * TL::QN;
    T *EB = EA + TL::EAW * TL::NE1;
    constexpr bool AUX1 = TL::template aux_own<T>();  // aux once per tile
    static_assert(AUX1 || RP::NA * TL::QN <= TL::EBW * TL::NE2, "cell aux area does not fit");
    static_assert(AUX1 || (RP::NUA == 0 && !RP::TNB),
                  "user aux and transverse-neighbour aux need the per-tile aux area");
    T *CA = AUX1 ? EB + TL::EBW * TL::NE2 : EB;
    const T tdtdx = (T)dtdx, tdtdy = (T)dtdy;

    load_tile<RP, T, TX, TY, NT>(a, qin, i0, j0, QS, CA);
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

    // both sweeps (the unsplit step), or one of them (a dimensionally split
    // step runs them as two launches, x first, with transverse_waves 0)
    const bool do_x = a.sweeps != 2, do_y = a.sweeps != 1;
    if (AUX1) {
        phase_aux<RP, T, 0, TX, TY, NT>(P, QS, CA);
        __syncthreads();
    }
    if (do_x) {
        if (!AUX1) {
            phase_aux<RP, T, 1, TX, TY, NT>(P, QS, CA);
            __syncthreads();
        }
        phase_rpn2<RP, T, 1, TX, TY, NT>(P, QS, CA, EA, i0, j0, a.mx, a.my, tdtdx, smax_x, bad);
        __syncthreads();
        phase_limit<RP, T, 1, TX, TY, NT>(P, EA, EB, CA, a.mthlim, a.order, a.tw, tdtdx);
        __syncthreads();
        phase_accum<RP, T, A, 1, TX, TY, NT, NC>(EA, EB, CA, acc, tdtdx, tdtdy);
        if (do_y) __syncthreads();
    }
    if (do_y) {
        if (!AUX1) {
            phase_aux<RP, T, 2, TX, TY, NT>(P, QS, CA);
            __syncthreads();
        }
        phase_rpn2<RP, T, 2, TX, TY, NT>(P, QS, CA, EA, i0, j0, a.mx, a.my, tdtdy, smax_y, bad);
        __syncthreads();
        phase_limit<RP, T, 2, TX, TY, NT>(P, EA, EB, CA, a.mthlim, a.order, a.tw, tdtdy);
        __syncthreads();
        phase_accum<RP, T, A, 2, TX, TY, NT, NC>(EA, EB, CA, acc, tdtdy, tdtdx);
    }

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


}  // namespace gclaw
