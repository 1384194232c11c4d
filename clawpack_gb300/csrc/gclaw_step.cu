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
#include "gclaw_pencil2.cuh"
#include "gclaw_step_impl.cuh"
#include "gclaw_strip.cuh"

#define GCLAW_VERSION_STR "gclaw 0.1.0 (sm_103a)"

namespace gclaw {

template <template <typename> class RPT, typename T, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, tile_min_blocks<T, NT>()) step_kernel(const StepArgs a,
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
    step_tile<RPT, T, TX, TY, NT>(a, P, qin, qout, dtdx, dtdy, blockIdx.x * TX,
                                  (blockIdx.y + a.ty0) * TY,
                                  smem_raw, smax_x, smax_y, bad);

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
            // with a capacity the tiles reduced Courant numbers, not speeds
            constexpr bool CN = RPT<T>::CAPA;
            if (a.no_finish) c->blocks_done = 0u;
            else finish_step(c, a.ctrl_mode, dt, CN ? 1.0 : dtdx, CN ? 1.0 : dtdy);
        }
    }
}

// FP32-bulk step over warp strips (gclaw_strip.cuh): one warp per strip of
// STRIP_W columns and seg_rows rows, units numbered strip-fastest so that
// the warps of a block work on neighbouring strips of the same rows.
#ifdef GCLAW_STRIP_MINB
#define GCLAW_STRIP_BLOCKS(RPT, T) GCLAW_STRIP_MINB
#else
#define GCLAW_STRIP_BLOCKS(RPT, T) strip_minb<RPT, T>()
#endif
template <template <typename> class RPT, typename T>
__global__ void __launch_bounds__(STRIP_NW * 32, GCLAW_STRIP_BLOCKS(RPT, T))
    strip_kernel(const StepArgs a, const typename RPT<T>::Params P, int seg_rows, int nstrips,
                 int nunits) {
    constexpr int NT = STRIP_NW * 32;
    constexpr bool RING = strip_ring<RPT, T>();
    extern __shared__ __align__(16) unsigned char strip_smem[];
    __shared__ double s_dt, s_dtdx, s_dtdy;
    __shared__ int s_par, s_skip;
    __shared__ T s_red[2][STRIP_NW];

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
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * STRIP_NW + (threadIdx.x >> 5);
    if (unit < nunits) {
        const int strip = unit % nstrips, seg = unit / nstrips;
        const int j0 = seg * seg_rows, j1 = min(j0 + seg_rows, a.my);
        T *ring = RING ? reinterpret_cast<T *>(strip_smem) +
                             (threadIdx.x >> 5) * 32 * strip_ring_floats<RPT<T>>()
                       : nullptr;
        strip_run<RPT, T, RING>(a, P, qin, qout, (T)dtdx, (T)dtdy, lane,
                                strip * STRIP_W + lane - 2, j0, j1, smax_x, smax_y, bad, ring);
    }

    const int anybad = block_reduce<T, NT>(smax_x, smax_y, bad, s_red);
    if (threadIdx.x == 0) {
        gclaw_ctrl *c = a.ctrl;
        atomicMax(&c->smax_bits[0], (unsigned long long)__double_as_longlong((double)smax_x));
        atomicMax(&c->smax_bits[1], (unsigned long long)__double_as_longlong((double)smax_y));
        if (anybad) atomicOr(&c->flags, 1u);
        __threadfence();
        const unsigned prev = atomicAdd(&c->blocks_done, 1u);
        if (prev == gridDim.x - 1) {
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
    dim3 grid((s->mx + TX - 1) / TX, a.nty > 0 ? a.nty : (s->my + TY - 1) / TY);
    for (int l = 0; l < nlaunch; l++) kern<<<grid, NT, smem, st>>>(a, P);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

// FP32-bulk kernel family: 0 = per-solver default, 1 = tiles, 2 = strips.
// The default is the faster family on GB300 at 2048^2: strips for all three
// solvers (acoustics 21.3 vs 14.0, shallow water 14.2 vs 12.2, Euler 9.1 vs
// 7.0 Gcell-updates/s); solvers that read transverse-neighbour aux run on
// tiles.
static int g_fp32_kernel = 0;
// FP64 kernel family: 0 = default (tiles), 1 = tiles, 2 = strips.
static int g_fp64_kernel = 0;
// Split-step kernel family: 0 = default (pencil sweeps, the y-sweep's kind
// per solver), 1 = tiles with a sweep mask, 2 = pencils with marching
// columns for the y-sweep, 3 = pencils with warp windows for both sweeps.
static int g_split_kernel = 0;

template <template <typename> class RPT, typename T>
static int launch_strip(const gclaw_solver *s, const StepArgs &a, cudaStream_t st, int nlaunch) {
    auto kern = strip_kernel<RPT, T>;
    constexpr size_t smem =
        strip_ring<RPT, T>() ? sizeof(T) * STRIP_NW * 32 * strip_ring_floats<RPT<T>>() : 0;
    static int warp_slots[32] = {0};  // resident warps per GPU, per device ordinal < 32
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GCLAW_ERR_CUDA;
    int slots = dev < 32 ? warp_slots[dev] : 0;
    if (slots == 0) {
        int nb = 0, nsm = 0;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess)
            return GCLAW_ERR_CUDA;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, STRIP_NW * 32, smem) !=
                cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return GCLAW_ERR_CUDA;
        slots = (nb > 0 ? nb : 1) * STRIP_NW * nsm;
        if (dev < 32) warp_slots[dev] = slots;
    }
    // row segments: enough strips x segments to fill the resident warps once,
    // without segments shorter than STRIP_MIN_ROWS rows
    const int nstrips = (s->mx + STRIP_W - 1) / STRIP_W;
    int nseg = slots / nstrips;
    if (nseg < 1) nseg = 1;
    int seg_rows = (s->my + nseg - 1) / nseg;
    if (seg_rows < STRIP_MIN_ROWS) seg_rows = STRIP_MIN_ROWS;
    nseg = (s->my + seg_rows - 1) / seg_rows;
    const int nunits = nstrips * nseg;
    const int nblocks = (nunits + STRIP_NW - 1) / STRIP_NW;
    const typename RPT<T>::Params P = RPT<T>::make(s->problem_data);
    for (int l = 0; l < nlaunch; l++)
        kern<<<nblocks, STRIP_NW * 32, smem, st>>>(a, P, seg_rows, nstrips, nunits);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

template <template <typename> class RPT>
static bool strip_default();
template <>
bool strip_default<RpAcoustics>() { return true; }
template <>
bool strip_default<RpShallow>() { return true; }
template <>
bool strip_default<RpEuler>() { return true; }

template <template <typename> class RPT, typename T>
static int launch_cfg(const gclaw_solver *s, const StepArgs &a, cudaStream_t st, int nlaunch) {
    using C = TileCfg<RPT, T>;
    // strips hold two rows of q only: no user aux, no transverse-neighbour aux
    if constexpr (!RPT<float>::TNB && RPT<float>::NUA == 0) {
        const bool split = a.sweeps == 1 || a.sweeps == 2;  // strips run both sweeps at once
        const bool strips = sizeof(T) == 4 ? (g_fp32_kernel == 2 ||
                                              (g_fp32_kernel == 0 && strip_default<RPT>()))
                                           : g_fp64_kernel == 2;
        if (strips && !split) return launch_strip<RPT, T>(s, a, st, nlaunch);
    }
    return launch_tile<RPT, T, C::TX, C::TY, C::NT>(s, a, st, nlaunch);
}

// Capacity variants: FP64 tiles of the solver wrapped in Capa.
template <template <typename> class RPT>
static int launch_capa(const gclaw_solver *s, const StepArgs &a, cudaStream_t st, int nlaunch) {
    using C = CapaTileCfg<RPT, double>;
    return launch_tile<Capa<RPT>::template rp, double, C::TX, C::TY, C::NT>(s, a, st, nlaunch);
}

// The product build's FP64 reciprocal over an array (gclaw_rcp_fp64).
__global__ void rcp_kernel(const double *__restrict__ x, double *__restrict__ y, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = qdiv(1.0, x[i]);
}

static int dispatch(const gclaw_solver *s, const StepArgs &a, cudaStream_t st, int nlaunch) {
    const bool f64 = s->precision == GCLAW_PREC_FP64;
    if (s->capa) {
        switch (s->rp) {
        case GCLAW_RP_ACOUSTICS_2D: return launch_capa<RpAcoustics>(s, a, st, nlaunch);
        case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D: return launch_capa<RpShallow>(s, a, st, nlaunch);
        case GCLAW_RP_EULER_4WAVE_2D: return launch_capa<RpEuler>(s, a, st, nlaunch);
        case GCLAW_RP_VC_ACOUSTICS_2D: return launch_capa<RpVcAcoustics>(s, a, st, nlaunch);
        case GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D:
            return launch_capa<RpShallowFwave>(s, a, st, nlaunch);
        default: return GCLAW_ERR_ARG;
        }
    }
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
    case GCLAW_RP_VC_ACOUSTICS_2D:
        return f64 ? launch_cfg<RpVcAcoustics, double>(s, a, st, nlaunch)
                   : launch_cfg<RpVcAcoustics, float>(s, a, st, nlaunch);
    case GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D:
        return f64 ? launch_cfg<RpShallowFwave, double>(s, a, st, nlaunch)
                   : launch_cfg<RpShallowFwave, float>(s, a, st, nlaunch);
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
    a.aux = (rp_user_aux(s->rp) || s->capa) ? s->aux : nullptr;
    a.maux = rp_num_aux(s->rp) + (s->capa ? 1 : 0);
    for (int d = 0; d < 2; d++) {
        a.abc_lo[d] = s->aux_bc_lower[d];
        a.abc_hi[d] = s->aux_bc_upper[d];
    }
}

// ---- host-buffer step, band by band ------------------------------------------
// gclaw_step_host moves a whole state each way every step.  For the FP64
// tile kernel the step is launched as GCLAW_HOST_BANDS bands of tile rows on
// the caller's stream while a copy stream moves the input rows in ahead of
// the band that needs them (its rows and the two-row halo) and the output
// rows of each finished band back, so the copies overlap the step except for
// the first input band and the last output band.  Bands other than the last
// leave the Courant reduction to the next (no_finish), so the result and the
// Courant number are those of one launch.
constexpr int GCLAW_HOST_BANDS = 4;

struct HostPipe {
    cudaStream_t copy;
    cudaEvent_t start, in[GCLAW_HOST_BANDS], done[GCLAW_HOST_BANDS], out;
    bool ready;
};
static HostPipe g_host_pipe[64];

// The copy stream and events of the current device, created on first use.
static int host_pipe(HostPipe **pp) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return GCLAW_ERR_CUDA;
    HostPipe &p = g_host_pipe[dev];
    if (!p.ready) {
        if (cudaStreamCreateWithFlags(&p.copy, cudaStreamNonBlocking) != cudaSuccess)
            return GCLAW_ERR_CUDA;
        cudaEvent_t *evs[] = {&p.start, &p.out};
        for (cudaEvent_t *e : evs)
            if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess)
                return GCLAW_ERR_CUDA;
        for (int b = 0; b < GCLAW_HOST_BANDS; b++)
            if (cudaEventCreateWithFlags(&p.in[b], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&p.done[b], cudaEventDisableTiming) != cudaSuccess)
                return GCLAW_ERR_CUDA;
        p.ready = true;
    }
    *pp = &p;
    return GCLAW_OK;
}

// Number of bands for this solver (1: one launch).  Banding needs the FP64
// tile kernel (the strip kernels cut rows their own way) and no periodic y
// boundary (whose halo rows come from the other end of the grid).
static int host_bands(const gclaw_solver *s) {
    if (s->precision != GCLAW_PREC_FP64 || g_fp64_kernel == 2 || s->capa) return 1;
    if (s->bc_lower[1] == GCLAW_BC_PERIODIC) return 1;
    int tx, ty;
    tile_shape(s->rp, s->precision, &tx, &ty);
    const int nty = (s->my + ty - 1) / ty;
    return nty >= 2 * GCLAW_HOST_BANDS ? GCLAW_HOST_BANDS : 1;
}

// Device addresses of pinned host arrays (both, or neither).
static void host_mapped(const double *q_host, double *qnew_host, const double **q_map,
                        double **new_map) {
    cudaPointerAttributes ai, ao;
    if (cudaPointerGetAttributes(&ai, q_host) != cudaSuccess ||
        cudaPointerGetAttributes(&ao, qnew_host) != cudaSuccess) {
        cudaGetLastError();  // clear the error state of the lookup
        return;
    }
    if (ai.type == cudaMemoryTypeHost && ao.type == cudaMemoryTypeHost && ai.devicePointer &&
        ao.devicePointer) {
        *q_map = (const double *)ai.devicePointer;
        *new_map = (double *)ao.devicePointer;
    }
}

static int step_host_banded(const gclaw_solver *s, const double *q_host, double *qnew_host,
                            double dt, double *d_q, double *d_new, gclaw_ctrl *ws,
                            cudaStream_t st, HostPipe *pp, int nband) {
    int m, mw, tx, ty;
    gclaw_rp_shape(s->rp, &m, &mw);
    tile_shape(s->rp, s->precision, &tx, &ty);
    const int nty = (s->my + ty - 1) / ty;
    const size_t row = (size_t)m * (size_t)s->mx;  // doubles per row of cells
    int t0[GCLAW_HOST_BANDS + 1];
    for (int b = 0; b <= nband; b++) t0[b] = (int)((long long)nty * b / nband);
    auto rows = [&](int b, size_t *off, size_t *n) {
        const int r0 = t0[b] * ty, r1 = t0[b + 1] * ty < s->my ? t0[b + 1] * ty : s->my;
        *off = row * (size_t)r0;
        *n = row * (size_t)(r1 - r0);
    };
    // the copy stream starts after the work already on the caller's stream
    if (cudaEventRecord(pp->start, st) != cudaSuccess ||
        cudaStreamWaitEvent(pp->copy, pp->start, 0) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    for (int b = 0; b < nband; b++) {
        size_t off, n;
        rows(b, &off, &n);
        if (cudaMemcpyAsync(d_q + off, q_host + off, n * sizeof(double),
                            cudaMemcpyHostToDevice, pp->copy) != cudaSuccess ||
            cudaEventRecord(pp->in[b], pp->copy) != cudaSuccess)
            return GCLAW_ERR_CUDA;
    }
    for (int b = 0; b < nband; b++) {
        // band b reads up to two rows past its end: the next band's input
        const int need = b + 1 < nband ? b + 1 : b;
        if (cudaStreamWaitEvent(st, pp->in[need], 0) != cudaSuccess) return GCLAW_ERR_CUDA;
        StepArgs a{};
        fill_args(s, a);
        a.qin[0] = a.qin[1] = d_q;
        a.qout[0] = a.qout[1] = d_new;
        a.ctrl = ws;
        a.dt = dt;
        a.ghosted = 0;
        a.ctrl_mode = 0;
        a.ty0 = t0[b];
        a.nty = t0[b + 1] - t0[b];
        a.no_finish = b + 1 < nband;
        int rc = dispatch(s, a, st, 1);
        if (rc) return rc;
        size_t off, n;
        rows(b, &off, &n);
        if (cudaEventRecord(pp->done[b], st) != cudaSuccess ||
            cudaStreamWaitEvent(pp->copy, pp->done[b], 0) != cudaSuccess ||
            cudaMemcpyAsync(qnew_host + off, d_new + off, n * sizeof(double),
                            cudaMemcpyDeviceToHost, pp->copy) != cudaSuccess)
            return GCLAW_ERR_CUDA;
    }
    if (cudaEventRecord(pp->out, pp->copy) != cudaSuccess ||
        cudaStreamWaitEvent(st, pp->out, 0) != cudaSuccess)
        return GCLAW_ERR_CUDA;
    return GCLAW_OK;
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
    case GCLAW_RP_VC_ACOUSTICS_2D: *num_eqn = 3; *num_waves = 2; return GCLAW_OK;
    case GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D: *num_eqn = 3; *num_waves = 3; return GCLAW_OK;
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
    if (s->capa) {
        // kappa is the field after the solver's own; FP64 only
        if (s->capa != rp_num_aux(s->rp) + 1 || !s->aux) return GCLAW_ERR_ARG;
        if (s->precision != GCLAW_PREC_FP64) return GCLAW_ERR_UNSUPPORTED;
        for (int d = 0; d < 2; d++) {
            if (s->aux_bc_lower[d] < GCLAW_BC_EXTRAP || s->aux_bc_lower[d] > GCLAW_BC_WALL ||
                s->aux_bc_upper[d] < GCLAW_BC_EXTRAP || s->aux_bc_upper[d] > GCLAW_BC_WALL)
                return GCLAW_ERR_ARG;
            if ((s->aux_bc_lower[d] == GCLAW_BC_PERIODIC) !=
                (s->aux_bc_upper[d] == GCLAW_BC_PERIODIC))
                return GCLAW_ERR_ARG;
        }
    }
    const double *pd = s->problem_data;
    switch (s->rp) {
    case GCLAW_RP_ACOUSTICS_2D:
        if (!(pd[2] > 0.0) || !(pd[3] > 0.0)) return GCLAW_ERR_ARG;
        break;
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D:
        if (!(pd[0] > 0.0)) return GCLAW_ERR_ARG;
        break;
    case GCLAW_RP_VC_ACOUSTICS_2D:
    case GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D:
        if (s->rp == GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D && !(pd[0] > 0.0)) return GCLAW_ERR_ARG;
        if (!s->aux) return GCLAW_ERR_ARG;
        for (int d = 0; d < 2; d++) {
            if (s->aux_bc_lower[d] < GCLAW_BC_EXTRAP || s->aux_bc_lower[d] > GCLAW_BC_WALL ||
                s->aux_bc_upper[d] < GCLAW_BC_EXTRAP || s->aux_bc_upper[d] > GCLAW_BC_WALL)
                return GCLAW_ERR_ARG;
            if ((s->aux_bc_lower[d] == GCLAW_BC_PERIODIC) !=
                (s->aux_bc_upper[d] == GCLAW_BC_PERIODIC))
                return GCLAW_ERR_ARG;
        }
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

int gclaw_fp32_kernel(int which) {
    const int prev = g_fp32_kernel;
    if (which >= 0 && which <= 2) g_fp32_kernel = which;
    return prev;
}

int gclaw_rcp_fp64(const double *x_dev, double *y_dev, long long n, void *stream) {
    if (!x_dev || !y_dev || n < 0) return GCLAW_ERR_ARG;
    if (n == 0) return GCLAW_OK;
    const unsigned nb = (unsigned)((n + 255) / 256);
    rcp_kernel<<<nb, 256, 0, (cudaStream_t)stream>>>(x_dev, y_dev, n);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

int gclaw_fp64_kernel(int which) {
    const int prev = g_fp64_kernel;
    if (which >= 0 && which <= 2) g_fp64_kernel = which;
    return prev;
}

int gclaw_split_kernel(int which) {
    const int prev = g_split_kernel;
    if (which >= 0 && which <= 3) g_split_kernel = which;
    return prev;
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

// state arrays of split steps start on 16 bytes (the pencil sweeps move
// cells of an even number of components as double2)
static bool al16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// Dimensionally split step: the x-sweep from qin into qtmp (its last block
// keeps the CFL reduction open), then the y-sweep from qtmp into qout, whose
// last block finishes the step with both sweeps' max |s|.
// Pencil sweeps (gclaw_pencil2.cuh) by default, for the solvers without
// aux; the tiles otherwise.
static int split_pencils(const gclaw_solver *s, const StepArgs &ax, const StepArgs &ay,
                         cudaStream_t st) {
    const bool f64 = s->precision == GCLAW_PREC_FP64;
    // y-sweep: warp windows for Euler (four components, 16-byte cells),
    // marching columns for the three-component solvers, whose windowed
    // y-loads touch twice the sectors (measured at 2048^2: acoustics FP32
    // 31.2 vs 17.2, Euler FP32 16.9 vs 17.9 Gcell-updates/s)
    const bool yw = g_split_kernel == 3 || (g_split_kernel == 0 && s->rp == GCLAW_RP_EULER_4WAVE_2D);
    switch (s->rp) {
    case GCLAW_RP_ACOUSTICS_2D:
        return f64 ? p2::split_step<RpAcoustics, double>(s, ax, ay, st, yw)
                   : p2::split_step<RpAcoustics, float>(s, ax, ay, st, yw);
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D:
        return f64 ? p2::split_step<RpShallow, double>(s, ax, ay, st, yw)
                   : p2::split_step<RpShallow, float>(s, ax, ay, st, yw);
    case GCLAW_RP_EULER_4WAVE_2D:
        return f64 ? p2::split_step<RpEuler, double>(s, ax, ay, st, yw)
                   : p2::split_step<RpEuler, float>(s, ax, ay, st, yw);
    default: return GCLAW_ERR_UNSUPPORTED;
    }
}

static int dispatch_split(const gclaw_solver *s, StepArgs ax, cudaStream_t st, int nsteps,
                          double *qtmp) {
    StepArgs ay = ax;
    ax.sweeps = 1;
    ax.no_finish = 1;
    ax.tw = 0;
    ax.qout[0] = ax.qout[1] = qtmp;
    ay.sweeps = 2;
    ay.no_finish = 0;
    ay.tw = 0;
    ay.qin[0] = ay.qin[1] = qtmp;
    for (int l = 0; l < nsteps; l++) {
        int rc = g_split_kernel != 1 ? split_pencils(s, ax, ay, st) : GCLAW_ERR_UNSUPPORTED;
        if (rc == GCLAW_ERR_UNSUPPORTED) {
            rc = dispatch(s, ax, st, 1);
            if (rc == GCLAW_OK) rc = dispatch(s, ay, st, 1);
        }
        if (rc != GCLAW_OK) return rc;
    }
    return GCLAW_OK;
}

int gclaw_step_split(const gclaw_solver *s, const double *q_dev, double *qnew_dev,
                     double *qtmp_dev, double dt, gclaw_ctrl *ws_dev, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!q_dev || !qnew_dev || !qtmp_dev || !ws_dev || !(dt > 0.0)) return GCLAW_ERR_ARG;
    if (rp_user_aux(s->rp) || s->capa) return GCLAW_ERR_UNSUPPORTED;
    if (qtmp_dev == q_dev || qtmp_dev == qnew_dev || q_dev == qnew_dev) return GCLAW_ERR_ARG;
    if (!al16(q_dev) || !al16(qnew_dev) || !al16(qtmp_dev)) return GCLAW_ERR_ARG;
    StepArgs a{};
    fill_args(s, a);
    a.qin[0] = a.qin[1] = q_dev;
    a.qout[0] = a.qout[1] = qnew_dev;
    a.ctrl = ws_dev;
    a.dt = dt;
    a.ghosted = 0;
    a.ctrl_mode = 0;
    return dispatch_split(s, a, (cudaStream_t)stream, 1, qtmp_dev);
}

int gclaw_advance_split(const gclaw_solver *s, double *q0_dev, double *q1_dev, double *qtmp_dev,
                        gclaw_ctrl *ctrl_dev, int nsteps, void *stream) {
    int rc = gclaw_check(s);
    if (rc) return rc;
    if (!q0_dev || !q1_dev || !qtmp_dev || !ctrl_dev || nsteps < 0) return GCLAW_ERR_ARG;
    if (rp_user_aux(s->rp) || s->capa) return GCLAW_ERR_UNSUPPORTED;
    if (qtmp_dev == q0_dev || qtmp_dev == q1_dev || q0_dev == q1_dev) return GCLAW_ERR_ARG;
    if (!al16(q0_dev) || !al16(q1_dev) || !al16(qtmp_dev)) return GCLAW_ERR_ARG;
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
    return dispatch_split(s, a, (cudaStream_t)stream, nsteps, qtmp_dev);
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
    // the workspace is raw caller memory: clear the control block whose
    // reduction slots and block counter the step expects at zero
    if (cudaMemsetAsync(ws, 0, sizeof(gclaw_ctrl), st) != cudaSuccess) return GCLAW_ERR_CUDA;
    // Pinned (page-locked) host arrays are addressable from the GPU: the step
    // then reads q and writes the new state through NVLink-C2C itself, with
    // no staging copy.  Other host memory goes through the device buffers.
    const double *q_map = nullptr;
    double *new_map = nullptr;
    host_mapped(q_host, qnew_host, &q_map, &new_map);
    HostPipe *pp = nullptr;
    const int nband = host_bands(s);
    if (q_map && new_map) {
        rc = gclaw_step(s, q_map, new_map, dt, ws, stream);
        if (rc) return rc;
    } else if (nband > 1 && host_pipe(&pp) == GCLAW_OK) {
        rc = step_host_banded(s, q_host, qnew_host, dt, d_q, d_new, ws, st, pp, nband);
        if (rc) return rc;
    } else {
        if (cudaMemcpyAsync(d_q, q_host, qb, cudaMemcpyHostToDevice, st) != cudaSuccess)
            return GCLAW_ERR_CUDA;
        rc = gclaw_step(s, d_q, d_new, dt, ws, stream);
        if (rc) return rc;
        if (cudaMemcpyAsync(qnew_host, d_new, qb, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return GCLAW_ERR_CUDA;
    }
    double cfl = 0.0;
    int status = 0;
    if (cudaMemcpyAsync(&cfl, &ws->cfl, sizeof(double), cudaMemcpyDeviceToHost, st) !=
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
__global__ void __launch_bounds__(NT, tile_min_blocks<T, NT>())
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
    step_tile<RPT, T, TX, TY, NT>(a, P, a.qin[0], a.qout[0], dtdx, dtdy, blockIdx.x * TX,
                                  blockIdx.y * TY, smem_raw, smax_x, smax_y, bad);
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
    if (s->capa) return GCLAW_ERR_UNSUPPORTED;
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
    case GCLAW_RP_VC_ACOUSTICS_2D: rc = GCLAW_LAUNCH_NA(RpVcAcoustics); break;
    case GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D: rc = GCLAW_LAUNCH_NA(RpShallowFwave); break;
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
