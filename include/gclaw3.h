/*
 * gclaw3.h -- C ABI of the classic unsplit 3D wave-propagation step on GB300.
 *
 * Replaces PyClaw's f2py call classic3.step3(...) for ClawSolver3D
 * (upstream pyclaw/src/pyclaw/classic/solver.py, step3.f90, flux3.f90;
 * empty submodules in the mounted clawpack 5.14.0 tree, meson.build:62-76)
 * with the Langseth-LeVeque method: per direction, normal Riemann solves,
 * limited correction fluxes, transverse splitting of the fluctuations in
 * both transverse directions and, with transverse_waves 11 or 22, the
 * corner (double transverse) terms.
 *
 * Arrays follow the f2py convention: q is (num_eqn, mx, my, mz) Fortran
 * order (component fastest).  The library allocates nothing: the caller
 * passes a device workspace of gclaw3_workspace_bytes() bytes and a
 * gclaw_ctrl block (include/gclaw.h), which also carries the time-step
 * control of gclaw3_advance.
 */
#ifndef GCLAW3_H
#define GCLAW3_H

#include <stddef.h>

#include "gclaw.h"

#ifdef __cplusplus
extern "C" {
#endif

/* acoustics_3D: m = 4 (p, u, v, w), 2 waves; pd: rho, bulk, cc, zz */
#define GCLAW3_RP_ACOUSTICS_3D 1
/* euler_3D: m = 5 (rho, rho u, rho v, rho w, E), 3 waves (acoustic, entropy
 * and shear together, acoustic), Roe, no entropy fix; pd: gamma */
#define GCLAW3_RP_EULER_3D 2

typedef struct gclaw3_solver {
    int rp;                       /* GCLAW3_RP_* */
    int mx, my, mz;               /* interior cells, each >= 2,
                                     (mx + 3)(my + 3)(mz + 3) < 2^31 */
    double dx, dy, dz;
    int bc_lower[3], bc_upper[3]; /* GCLAW_BC_EXTRAP / PERIODIC / WALL per axis */
    int mthlim[GCLAW_MAX_WAVES];  /* limiter per wave family */
    int order;                    /* 1 or 2 */
    int transverse_waves;         /* 0, 10, 11, 20 or 22 (ClawSolver3D: 22) */
    int precision;                /* GCLAW_PREC_FP64, or GCLAW_PREC_FP32_BULK: FP32 edge
                                     records and fluxes, FP64 state */
    double problem_data[8];
} gclaw3_solver;

int gclaw3_rp_shape(int rp, int *num_eqn, int *num_waves);

/* 0 if the description can be stepped, else GCLAW_ERR_ARG or
 * GCLAW_ERR_UNSUPPORTED (unknown transverse option or precision). */
int gclaw3_check(const gclaw3_solver *s);

/* Bytes of device workspace a step of this grid needs. */
size_t gclaw3_workspace_bytes(const gclaw3_solver *s);

/* State arrays (q_dev, qnew_dev, q0_dev, q1_dev, qtmp_dev) start on a
 * 16-byte boundary, as cudaMalloc returns them; others are refused with
 * GCLAW_ERR_ARG. */

/* One step of size dt from q_dev into qnew_dev (interior arrays, distinct).
 * ctrl_dev receives the Courant number (cfl) and status (GCLAW_OK or
 * GCLAW_NONPHYSICAL); only its reduction fields are used.  Asynchronous on
 * stream. */
int gclaw3_step(const gclaw3_solver *s, const double *q_dev, double *qnew_dev, double dt,
                void *ws_dev, gclaw_ctrl *ctrl_dev, void *stream);

/* nsteps attempts under device time-step control (gclaw_ctrl_init first):
 * the state ping-pongs between q0_dev and q1_dev, ctrl->parity names the
 * accepted one; rejected attempts and finished runs are skipped on the
 * device.  Capturable in a CUDA graph. */
int gclaw3_advance(const gclaw3_solver *s, double *q0_dev, double *q1_dev, void *ws_dev,
                   gclaw_ctrl *ctrl_dev, int nsteps, void *stream);

/* PyClaw's dimensionally split 3D step (ClawSolver3D with
 * dimensional_split = True, its default; classic3 step3ds): the x-, y- and
 * z-sweeps in turn, each from the previous one's result with the boundary
 * conditions applied to it, without transverse terms (transverse_waves is
 * ignored); qtmp_dev is a third state buffer, distinct from the others.
 * The Courant number is the largest of the three sweeps'.  Split sweeps
 * keep no edge records: ws_dev is not used and may be NULL. */
int gclaw3_step_split(const gclaw3_solver *s, const double *q_dev, double *qnew_dev,
                      double *qtmp_dev, double dt, void *ws_dev, gclaw_ctrl *ctrl_dev,
                      void *stream);
int gclaw3_advance_split(const gclaw3_solver *s, double *q0_dev, double *q1_dev,
                         double *qtmp_dev, void *ws_dev, gclaw_ctrl *ctrl_dev, int nsteps,
                         void *stream);

/* Kernel of the sweeps without transverse terms (split steps, and
 * transverse_waves 0) along y and z: 0 = default (threads marching along
 * the pencil), 1 = marching, 2 = warp windows across the pencil.  The
 * x-sweep always runs on warp windows.  Bit-identical with -fmad=false.
 * Returns the previous setting. */
int gclaw3_split_kernel(int which);

/* Kernels of the sweeps with transverse terms: 0 = default (FP32-bulk: one
 * fused kernel per sweep, the chains exchanged in shared memory; FP64: the
 * three staged kernels through the workspace), 1 = the staged kernels.
 * Bit-identical with -fmad=false.  Returns the previous setting. */
int gclaw3_unsplit_kernel(int which);

#ifdef __cplusplus
}
#endif

#endif
