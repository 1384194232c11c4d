// gclaw_batch.cu -- many independent classic 2D problems advanced together.
//
// Thousands of problems of uneven grid sizes share one solver description
// (Riemann solver, boundary conditions, limiters, precision) and have their
// own grid, cell sizes and time-step control.  Their states live in two
// large FP64 buffers (q0, q1), problem p at offset q_offset[p], each in the
// (num_eqn, mx, my) Fortran layout of a single problem.
//
// One launch is one attempted step of every unfinished problem.  FP64
// (batch_step_kernel): a persistent grid of CTAs strides over all tiles of
// all problems; a CTA finds the problem of its tile by binary search over
// the tiles' prefix sums and runs the single-problem tile body.  FP32-bulk
// (batch_strip_kernel): a persistent grid of warps strides over all strip
// units (problem, 28-column strip, 64-row segment) and runs the
// single-problem strip body, which needs no barriers and suits small
// problems.  Either way each problem's result is bit-identical to stepping
// it alone, and each unit feeds the problem's CFL reduction.  The last unit
// of a problem to finish applies PyClaw's evolve_to_time rules to that
// problem's gclaw_ctrl (accept / reject, dt from its own CFL, stop after
// max_accepted steps).  N steps are N launches, which capture into one CUDA
// graph.  The table and the control blocks are caller-owned device memory.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gclaw.h"
#include "gclaw_step_impl.cuh"
#include "gclaw_strip.cuh"

namespace gclaw {

// One problem of the device table (48 bytes): its tile decomposition (tile
// kernels) and its strip decomposition (FP32 strip kernels: strips of
// STRIP_W columns times segments of BATCH_SEG rows).
struct BatchEntry {
    int mx, my;
    int tiles_x, ntiles;
    double dx, dy;
    long long q_off;
    int strips_x, nunits;
};
constexpr int BATCH_SEG = 64;

// Batched FP32-bulk steps on warp strips: a persistent grid of warps strides
// over the strip units (problem, strip, row segment) of all problems; a warp
// finds the problem of its unit by probing the units' prefix sums forward
// from the problem of its previous unit (its units only increase), marches
// the unit exactly as the single-problem strip kernel does (so a problem's
// result does not depend on being batched), reduces max |s| across its lanes
// into the problem's control block, and the problem's last unit applies the
// evolve_to_time rules.
template <template <typename> class RPT>
__global__ void __launch_bounds__(STRIP_NW * 32, StripCfg<RPT>::MINB)
    batch_strip_kernel(const StepArgs base, const typename RPT<float>::Params P,
                       const BatchEntry *__restrict__ ent, const int *__restrict__ ustart,
                       int nprob, double *q0, double *q1, gclaw_ctrl *ctrls) {
    constexpr bool RING = strip_ring<RPT, float>();
    extern __shared__ __align__(16) unsigned char strip_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nw = gridDim.x * STRIP_NW;
    const int total = __ldg(ustart + nprob);
    float *ring = RING ? reinterpret_cast<float *>(strip_smem) +
                             wib * 32 * strip_ring_floats<RPT<float>>()
                       : nullptr;
    int pcur = 0;
    for (int u = blockIdx.x * STRIP_NW + wib; u < total; u += nw) {
        int lo = pcur;  // largest p with ustart[p] <= u
        for (;;) {
            const int idx = lo + 1 + lane;
            const bool le = idx < nprob && __ldg(ustart + idx) <= u;
            const int c = __popc(__ballot_sync(0xffffffffu, le));
            lo += c;
            if (c < 32) break;
        }
        pcur = lo;
        gclaw_ctrl *c = ctrls + lo;
        int done = 0, par = 0;
        double dt = 0.0;
        if (lane == 0) {
            const volatile gclaw_ctrl *vc = c;
            done = vc->done;
            par = vc->parity;
            dt = vc->dt;
        }
        done = __shfl_sync(0xffffffffu, done, 0);
        if (done) continue;
        par = __shfl_sync(0xffffffffu, par, 0);
        dt = __shfl_sync(0xffffffffu, dt, 0);
        const BatchEntry e = ent[lo];
        StepArgs a = base;
        a.mx = e.mx;
        a.my = e.my;
        a.dx = e.dx;
        a.dy = e.dy;
        double *qa = q0 + e.q_off, *qb = q1 + e.q_off;
        const double *qin = par ? qb : qa;
        double *qout = par ? qa : qb;
        const int local = u - __ldg(ustart + lo);
        const int strip = local % e.strips_x, seg = local / e.strips_x;
        const int j0 = seg * BATCH_SEG, j1 = min(j0 + BATCH_SEG, e.my);
        const double dtdx = dt / e.dx, dtdy = dt / e.dy;
        float smax_x = 0.0f, smax_y = 0.0f;
        bool bad = false;
        strip_run<RPT, float, RING>(a, P, qin, qout, (float)dtdx, (float)dtdy, lane,
                                    strip * STRIP_W + lane - 2, j0, j1, smax_x, smax_y, bad,
                                    ring);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            smax_x = fmaxf(smax_x, __shfl_xor_sync(0xffffffffu, smax_x, off));
            smax_y = fmaxf(smax_y, __shfl_xor_sync(0xffffffffu, smax_y, off));
        }
        const bool anybad = __any_sync(0xffffffffu, bad);
        if (lane == 0) {
            atomicMax(&c->smax_bits[0], (unsigned long long)__double_as_longlong((double)smax_x));
            atomicMax(&c->smax_bits[1], (unsigned long long)__double_as_longlong((double)smax_y));
            if (anybad) atomicOr(&c->flags, 1u);
            __threadfence();
            if (atomicAdd(&c->blocks_done, 1u) == (unsigned)e.nunits - 1u) {
                __threadfence();
                finish_step(c, 1, dt, dtdx, dtdy);
            }
        }
    }
}

template <template <typename> class RPT, typename T, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, tile_min_blocks<T, NT>())
    batch_step_kernel(const StepArgs base, const typename RPT<T>::Params P,
                      const BatchEntry *__restrict__ ent, const int *__restrict__ tstart,
                      int nprob, int total_tiles, double *q0, double *q1, gclaw_ctrl *ctrls) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double s_dt, s_dtdx, s_dtdy;
    __shared__ int s_p, s_par, s_skip;
    __shared__ T s_red[2][NT / 32];

    for (int t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        if (threadIdx.x == 0) {
            int lo = 0, hi = nprob;  // largest p with tstart[p] <= t
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (__ldg(tstart + mid) <= t) lo = mid;
                else hi = mid;
            }
            const volatile gclaw_ctrl *c = ctrls + lo;
            const double dt = c->dt;
            s_p = lo;
            s_skip = c->done;
            s_par = c->parity;
            s_dt = dt;
            s_dtdx = dt / ent[lo].dx;
            s_dtdy = dt / ent[lo].dy;
        }
        __syncthreads();
        if (!s_skip) {
            const int p = s_p;
            const BatchEntry e = ent[p];
            StepArgs a = base;
            a.mx = e.mx;
            a.my = e.my;
            a.dx = e.dx;
            a.dy = e.dy;
            double *qa = q0 + e.q_off, *qb = q1 + e.q_off;
            const double *qin = s_par ? qb : qa;
            double *qout = s_par ? qa : qb;
            const int local = t - __ldg(tstart + p);
            const int ti = local % e.tiles_x, tj = local / e.tiles_x;
            const double dt = s_dt, dtdx = s_dtdx, dtdy = s_dtdy;
            T smax_x = (T)0, smax_y = (T)0;
            bool bad = false;
            step_tile<RPT, T, TX, TY, NT>(a, P, qin, qout, dtdx, dtdy, ti * TX, tj * TY, smem_raw,
                                          smax_x, smax_y, bad);
            const int anybad = block_reduce<T, NT>(smax_x, smax_y, bad, s_red);
            if (threadIdx.x == 0) {
                gclaw_ctrl *c = ctrls + p;
                atomicMax(&c->smax_bits[0], (unsigned long long)__double_as_longlong((double)smax_x));
                atomicMax(&c->smax_bits[1], (unsigned long long)__double_as_longlong((double)smax_y));
                if (anybad) atomicOr(&c->flags, 1u);
                __threadfence();
                if (atomicAdd(&c->blocks_done, 1u) == (unsigned)e.ntiles - 1u) {
                    __threadfence();
                    finish_step(c, 1, dt, dtdx, dtdy);
                }
            }
        }
        __syncthreads();  // shared memory is reused by the next tile
    }
}

__global__ void batch_ctrl_init_kernel(gclaw_ctrl *c, int nprob, const double *dt0, double t,
                                       double t_end, double cfl_max, double cfl_desired,
                                       double dt_max, int max_steps, int max_accepted,
                                       int dt_variable) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    double dt = dt0[p];
    if (t + dt > t_end && t < t_end) dt = t_end - t;
    if (t_end - t - dt < 1.0e-14 * t) dt = t_end - t;
    gclaw_ctrl z;
    memset(&z, 0, sizeof z);
    z.t = t;
    z.dt = dt;
    z.t_start = t;
    z.t_end = t_end;
    z.cfl_max = cfl_max;
    z.cfl_desired = cfl_desired;
    z.dt_max = dt_max;
    z.dtmin = dt;
    z.dtmax = dt;
    z.max_steps = max_steps;
    z.max_accepted = max_accepted;
    z.dt_variable = dt_variable;
    z.done = (t >= t_end) ? 1 : 0;
    z.status = GCLAW_OK;
    c[p] = z;
}

template <template <typename> class RPT, typename T>
static int launch_batch(const gclaw_solver *s, const StepArgs &a, const void *table, int nprob,
                        int total_tiles, double *q0, double *q1, gclaw_ctrl *ctrls, int nlaunch,
                        cudaStream_t st) {
    using C = TileCfg<RPT, T>;
    using RP = RPT<T>;
    using TL = Tile<RP, C::TX, C::TY>;
    constexpr size_t smem = TL::template smem_bytes<T>();
    auto kern = batch_step_kernel<RPT, T, C::TX, C::TY, C::NT>;
    static int grid_of_dev[64];  // persistent grid size per device, 0 = not yet set up
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return GCLAW_ERR_CUDA;
    if (grid_of_dev[dev] == 0) {
        int sms = 0, per_sm = 0;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, smem) !=
                cudaSuccess ||
            per_sm < 1)
            return GCLAW_ERR_CUDA;
        grid_of_dev[dev] = sms * per_sm;
    }
    const int grid = total_tiles < grid_of_dev[dev] ? total_tiles : grid_of_dev[dev];
    const BatchEntry *ent = (const BatchEntry *)table;
    const int *tstart = (const int *)((const char *)table + sizeof(BatchEntry) * (size_t)nprob);
    const typename RP::Params P = RP::make(s->problem_data);
    for (int l = 0; l < nlaunch; l++)
        kern<<<grid, C::NT, smem, st>>>(a, P, ent, tstart, nprob, total_tiles, q0, q1, ctrls);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

template <template <typename> class RPT>
static int launch_batch_strip(const gclaw_solver *s, const StepArgs &a, const void *table,
                              int nprob, double *q0, double *q1, gclaw_ctrl *ctrls, int nlaunch,
                              cudaStream_t st) {
    auto kern = batch_strip_kernel<RPT>;
    constexpr size_t smem =
        strip_ring<RPT, float>() ? sizeof(float) * STRIP_NW * 32 * strip_ring_floats<RPT<float>>()
                                 : 0;
    static int grid_of_dev[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return GCLAW_ERR_CUDA;
    if (grid_of_dev[dev] == 0) {
        int sms = 0, per_sm = 0;
        if ((smem > 48 * 1024 &&
             cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                 cudaSuccess) ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, STRIP_NW * 32, smem) !=
                cudaSuccess ||
            per_sm < 1)
            return GCLAW_ERR_CUDA;
        grid_of_dev[dev] = sms * per_sm;
    }
    const BatchEntry *ent = (const BatchEntry *)table;
    const int *ustart = (const int *)((const char *)table + sizeof(BatchEntry) * (size_t)nprob +
                                      sizeof(int) * ((size_t)nprob + 1));
    const typename RPT<float>::Params P = RPT<float>::make(s->problem_data);
    for (int l = 0; l < nlaunch; l++)
        kern<<<grid_of_dev[dev], STRIP_NW * 32, smem, st>>>(a, P, ent, ustart, nprob, q0, q1,
                                                            ctrls);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

// gclaw_check on the shared part of a batch's solver description (the
// per-problem grid fields are ignored).
static int check_shared(const gclaw_solver *s) {
    if (!s) return GCLAW_ERR_ARG;
    gclaw_solver c = *s;
    c.mx = c.my = 2;
    c.dx = c.dy = 1.0;
    return gclaw_check(&c);
}

}  // namespace gclaw

using namespace gclaw;

extern "C" {

size_t gclaw_batch_table_bytes(int nprob) {
    if (nprob < 1) return 0;
    return sizeof(BatchEntry) * (size_t)nprob + 2 * sizeof(int) * ((size_t)nprob + 1);
}

int gclaw_batch_prepare(const gclaw_solver *s, const gclaw_batch_problem *probs, int nprob,
                        void *table_dev, size_t table_bytes, int *total_tiles, void *stream) {
    int rc = check_shared(s);
    if (rc) return rc;
    if (!probs || nprob < 1 || !table_dev || !total_tiles) return GCLAW_ERR_ARG;
    if (table_bytes < gclaw_batch_table_bytes(nprob)) return GCLAW_ERR_WORKSPACE;
    if (((uintptr_t)table_dev & 15u) != 0) return GCLAW_ERR_ARG;
    int tx, ty;
    tile_shape(s->rp, s->precision, &tx, &ty);
    const size_t nbytes = gclaw_batch_table_bytes(nprob);
    unsigned char *host = (unsigned char *)malloc(nbytes);
    if (!host) return GCLAW_ERR_ARG;
    BatchEntry *ent = (BatchEntry *)host;
    int *tstart = (int *)(host + sizeof(BatchEntry) * (size_t)nprob);
    int *ustart = tstart + nprob + 1;
    long long tiles = 0, units = 0;
    for (int p = 0; p < nprob; p++) {
        const gclaw_batch_problem &b = probs[p];
        if (b.mx < 2 || b.my < 2 || !(b.dx > 0.0) || !(b.dy > 0.0) || b.q_offset < 0) {
            free(host);
            return GCLAW_ERR_ARG;
        }
        ent[p].mx = b.mx;
        ent[p].my = b.my;
        ent[p].tiles_x = (b.mx + tx - 1) / tx;
        ent[p].ntiles = ent[p].tiles_x * ((b.my + ty - 1) / ty);
        ent[p].dx = b.dx;
        ent[p].dy = b.dy;
        ent[p].q_off = b.q_offset;
        ent[p].strips_x = (b.mx + STRIP_W - 1) / STRIP_W;
        ent[p].nunits = ent[p].strips_x * ((b.my + BATCH_SEG - 1) / BATCH_SEG);
        tstart[p] = (int)tiles;
        ustart[p] = (int)units;
        tiles += ent[p].ntiles;
        units += ent[p].nunits;
        if (tiles > 0x7fffffffll || units > 0x7fffffffll) {
            free(host);
            return GCLAW_ERR_ARG;
        }
    }
    tstart[nprob] = (int)tiles;
    ustart[nprob] = (int)units;
    cudaStream_t st = (cudaStream_t)stream;
    const bool ok = cudaMemcpyAsync(table_dev, host, nbytes, cudaMemcpyHostToDevice, st) ==
                        cudaSuccess &&
                    cudaStreamSynchronize(st) == cudaSuccess;
    free(host);
    if (!ok) return GCLAW_ERR_CUDA;
    *total_tiles = (int)tiles;
    return GCLAW_OK;
}

int gclaw_batch_ctrl_init(gclaw_ctrl *ctrls_dev, int nprob, const double *dt0_dev, double t,
                          double t_end, double cfl_max, double cfl_desired, double dt_max,
                          int max_steps, int max_accepted, int dt_variable, void *stream) {
    if (!ctrls_dev || !dt0_dev || nprob < 1 || max_steps < 1) return GCLAW_ERR_ARG;
    batch_ctrl_init_kernel<<<(nprob + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        ctrls_dev, nprob, dt0_dev, t, t_end, cfl_max, cfl_desired, dt_max, max_steps,
        max_accepted, dt_variable ? 1 : 0);
    return cudaGetLastError() == cudaSuccess ? GCLAW_OK : GCLAW_ERR_CUDA;
}

int gclaw_batch_advance(const gclaw_solver *s, const void *table_dev, int nprob, int total_tiles,
                        double *q0_dev, double *q1_dev, gclaw_ctrl *ctrls_dev, int nlaunch,
                        void *stream) {
    int rc = check_shared(s);
    if (rc) return rc;
    if (!table_dev || nprob < 1 || total_tiles < 1 || !q0_dev || !q1_dev || !ctrls_dev ||
        nlaunch < 0)
        return GCLAW_ERR_ARG;
    StepArgs a{};
    a.ghosted = 0;
    a.ctrl_mode = 1;
    for (int d = 0; d < 2; d++) {
        a.bc_lo[d] = s->bc_lower[d];
        a.bc_hi[d] = s->bc_upper[d];
    }
    a.mthlim = 0;
    for (int p = 0; p < 4; p++) a.mthlim |= (s->mthlim[p] & 0xff) << (8 * p);
    a.order = s->order;
    a.tw = s->transverse_waves;
    cudaStream_t st = (cudaStream_t)stream;
    const bool f64 = s->precision == GCLAW_PREC_FP64;
    // FP32-bulk runs on strips unless tiles were selected for the process
    // (the same choice as for single problems, so batched and single runs
    // of a problem agree bit for bit)
    const int fam = gclaw_fp32_kernel(-1);
    if (rp_user_aux(s->rp) || s->capa) return GCLAW_ERR_UNSUPPORTED;  // no per-problem aux
    if (!f64 && fam != 1) {
        switch (s->rp) {
        case GCLAW_RP_ACOUSTICS_2D:
            return launch_batch_strip<RpAcoustics>(s, a, table_dev, nprob, q0_dev, q1_dev,
                                                   ctrls_dev, nlaunch, st);
        case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D:
            return launch_batch_strip<RpShallow>(s, a, table_dev, nprob, q0_dev, q1_dev,
                                                 ctrls_dev, nlaunch, st);
        default:
            return launch_batch_strip<RpEuler>(s, a, table_dev, nprob, q0_dev, q1_dev, ctrls_dev,
                                               nlaunch, st);
        }
    }
#define GCLAW_BATCH(RPT)                                                                         \
    (f64 ? launch_batch<RPT, double>(s, a, table_dev, nprob, total_tiles, q0_dev, q1_dev,       \
                                     ctrls_dev, nlaunch, st)                                     \
         : launch_batch<RPT, float>(s, a, table_dev, nprob, total_tiles, q0_dev, q1_dev,        \
                                    ctrls_dev, nlaunch, st))
    switch (s->rp) {
    case GCLAW_RP_ACOUSTICS_2D: return GCLAW_BATCH(RpAcoustics);
    case GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D: return GCLAW_BATCH(RpShallow);
    default: return GCLAW_BATCH(RpEuler);
    }
#undef GCLAW_BATCH
}

}  // extern "C"
