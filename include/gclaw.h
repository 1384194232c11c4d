/*
 * gclaw.h -- C ABI of libgclaw.so, the GB300 (sm_103a) classic unsplit 2D
 * wave-propagation step.
 *
 * The reference path this replaces is PyClaw's ClawSolver2D.step() calling
 * the f2py module classic2.step2(...) with the rpn2/rpt2 callbacks of a
 * clawpack.riemann module (upstream pyclaw/src/pyclaw/classic/solver.py and
 * step2.f90; the submodules are empty in the mounted umbrella tree,
 * .gitmodules:1-21, and are mapped by meson.build:62-76).  The f2py array
 * convention is kept: q is (num_eqn, mx, my) in Fortran order, i.e. the
 * component index varies fastest, then x, then y.  With ghost cells it is
 * PyClaw's qbc, (num_eqn, mx+4, my+4) for num_ghost = 2.
 *
 * Conventions
 *   - Every pointer named *_dev is device memory owned by the caller; the
 *     library allocates nothing and only borrows pointers.
 *   - stream is a cudaStream_t passed as void* (NULL = legacy stream).
 *   - Return value: 0 = GCLAW_OK, < 0 argument / CUDA errors, > 0 numerical
 *     conditions (non-physical state, CFL rejection with fixed dt, step cap).
 *   - One gclaw_ctrl per concurrently advancing problem; calls that share a
 *     gclaw_ctrl must be ordered on one stream.
 */
#ifndef GCLAW_H
#define GCLAW_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Riemann solvers: the clawpack.riemann modules of the same name
 * (conda-recipe/meta.yaml:36 imports clawpack.riemann.euler_4wave_2D). */
#define GCLAW_RP_ACOUSTICS_2D 1             /* m=3 (p,u,v), 2 waves; pd: rho, bulk, cc, zz */
#define GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D 2 /* m=3 (h,hu,hv), 3 waves; pd: grav */
#define GCLAW_RP_EULER_4WAVE_2D 3           /* m=4 (rho,rhou,rhov,E), 4 waves; pd: gamma, efix */
#define GCLAW_RP_VC_ACOUSTICS_2D 4          /* m=3 (p,u,v), 2 waves; aux (rho, c) per cell */
/* shallow_bathymetry_fwave_2D: m=3 (h,hu,hv), 3 f-waves; aux (b) per cell, the
 * bottom elevation; pd: grav.  Depths must stay positive (no dry cells). */
#define GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D 5

/* Boundary conditions: the values of pyclaw.BC. */
#define GCLAW_BC_CUSTOM 0 /* not supported: rejected with GCLAW_ERR_UNSUPPORTED */
#define GCLAW_BC_EXTRAP 1
#define GCLAW_BC_PERIODIC 2
#define GCLAW_BC_WALL 3

/* Wave limiters: the values of pyclaw.limiters.tvd. */
#define GCLAW_LIM_NONE 0
#define GCLAW_LIM_MINMOD 1
#define GCLAW_LIM_SUPERBEE 2
#define GCLAW_LIM_VANLEER 3
#define GCLAW_LIM_MC 4

/* Arithmetic of the flux computation.  Storage of q is FP64 in both. */
#define GCLAW_PREC_FP64 0      /* plain FP64, the drop-in for the Fortran step */
#define GCLAW_PREC_FP32_BULK 1 /* FP32 waves/fluxes, FP64 accumulation and CFL */

/* Status codes. */
#define GCLAW_OK 0
#define GCLAW_ERR_ARG (-1)
#define GCLAW_ERR_CUDA (-2)
#define GCLAW_ERR_UNSUPPORTED (-4)
#define GCLAW_ERR_WORKSPACE (-5)
#define GCLAW_ERR_TOO_LARGE (-6) /* grid exceeds GCLAW_NOALLOC_MAX_BLOCKS thread blocks */
#define GCLAW_NONPHYSICAL 2  /* NaN Courant number or negative Euler c^2 */
#define GCLAW_CFL_FIXED_DT 3 /* step rejected while dt_variable = 0 */
#define GCLAW_MAX_STEPS 4    /* attempts reached max_steps before tend */

#define GCLAW_MAX_WAVES 4

/* Solver description: the attributes of pyclaw.ClawSolver2D that the step
 * reads, plus the grid.  mx, my >= 2; num_ghost is fixed at 2. */
typedef struct gclaw_solver {
    int rp;                       /* GCLAW_RP_* */
    int mx, my;                   /* interior cells */
    double dx, dy;                /* cell sizes */
    int bc_lower[2], bc_upper[2]; /* GCLAW_BC_* for x and y */
    int mthlim[GCLAW_MAX_WAVES];  /* limiter per wave family (solver.limiters) */
    int order;                    /* 1 or 2 (solver.order) */
    int transverse_waves;         /* 0, 1 or 2 (solver.transverse_waves) */
    int precision;                /* GCLAW_PREC_* */
    double problem_data[8];       /* state.problem_data, layout per GCLAW_RP_* */
    /* Solvers with an aux array (GCLAW_RP_VC_ACOUSTICS_2D, maux = 2;
     * GCLAW_RP_SHALLOW_BATHYMETRY_FWAVE_2D, maux = 1): device pointer to
     * aux, laid out like q with maux components -- (maux, mx, my), or
     * (maux, mx+4, my+4) with ghost cells filled for gclaw_step2 -- and its
     * boundary conditions (state.aux; solver.aux_bc_lower / aux_bc_upper;
     * walls mirror without negation).  Ignored by the other solvers; a
     * zero-initialised tail means "no aux". */
    const double *aux;
    int aux_bc_lower[2], aux_bc_upper[2];
    /* Capacity function (classic2's mcapa = state.index_capa + 1): 0 for
     * none, else the 1-based index of the capacity field kappa in aux, which
     * must be the field after the solver's own (maux = solver's + 1; for
     * the solvers without aux, aux holds kappa alone).  The step then takes
     * dt / (kappa dx) per cell and divides each cell's flux differences by
     * its kappa.  FP64, unsplit steps with a workspace (gclaw_step,
     * gclaw_step2, gclaw_advance and their host forms); refused with
     * GCLAW_ERR_UNSUPPORTED elsewhere. */
    int capa;
} gclaw_solver;

/* Time-step control block, resident in device memory.  The step kernel's
 * last block applies PyClaw's evolve_to_time rules to it (upstream
 * pyclaw/src/pyclaw/solver.py): reject when cfl > cfl_max, otherwise
 * t += dt; then dt = min(dt_max, dt*cfl_desired/cfl), clipped to land on
 * t_end.  Fields marked (in) are set by the caller before advancing. */
typedef struct gclaw_ctrl {
    double t;            /* time of the accepted state (in/out) */
    double dt;           /* dt of the next attempt (in/out) */
    double t_start;      /* time at the start of this evolve call (in) */
    double t_end;        /* stop when t >= t_end (in) */
    double cfl_max;      /* (in) */
    double cfl_desired;  /* (in) */
    double dt_max;       /* (in) */
    double cfl;          /* Courant number of the last attempt (out) */
    double cflmax;       /* largest accepted Courant number (out) */
    double dtmin, dtmax; /* range of dt chosen (out) */
    unsigned long long smax_bits[2]; /* scratch: max |s| of x and y edges */
    int parity;          /* buffer holding the accepted state, 0 or 1 (in/out) */
    int numsteps;        /* accepted steps (out) */
    int attempts;        /* attempted steps (out) */
    int max_steps;       /* cap on attempts, PyClaw's solver.max_steps (in) */
    int max_accepted;    /* stop after this many accepted steps; < 0: none (in) */
    int dt_variable;     /* 1 (default) or 0 (in) */
    int done;            /* 1 once finished or failed (out) */
    int status;          /* GCLAW_OK or a positive status (out) */
    unsigned int blocks_done; /* scratch: last-block counter */
    unsigned int flags;       /* scratch: non-physical flag of this attempt */
} gclaw_ctrl;

/* Library version string. */
const char *gclaw_version(void);

/* Text for a status code. */
const char *gclaw_strerror(int status);

/* Number of equations and waves of a Riemann solver id (0 on success). */
int gclaw_rp_shape(int rp, int *num_eqn, int *num_waves);

/* Validate a solver description (0 if it can be stepped). */
int gclaw_check(const gclaw_solver *s);

/* Set a control block to its initial state on stream: t, dt, t_end, the
 * PyClaw controls, parity 0, counters zero.  max_accepted < 0 disables the
 * step-count stop; dt is clipped to t_end as PyClaw does before a step.
 * The fields are written by a one-thread kernel enqueued on stream, so the
 * call neither copies from host memory nor synchronises, and can be
 * captured in a CUDA graph. */
int gclaw_ctrl_init(gclaw_ctrl *ctrl_dev, double t, double dt, double t_end, double cfl_max,
                    double cfl_desired, double dt_max, int max_steps, int max_accepted,
                    int dt_variable, void *stream);

/* Kernel family of the FP32-bulk step, for the whole process: 0 = the
 * per-solver default, 1 = shared-memory tiles, 2 = register strips (one
 * warp per 28-column strip marching up its rows).  Both compute the same
 * step; any other value only queries.  Returns the previous setting. */
int gclaw_fp32_kernel(int which);

/* The same for the FP64 step: 0 = default (tiles), 1 = tiles, 2 = register
 * strips (bit-identical to tiles with -fmad=false). */
int gclaw_fp64_kernel(int which);

/* Kernel family of the dimensionally split step: 0 = default (one pencil
 * kernel per sweep: warp windows along x; along y threads marching up
 * columns, or warp windows for euler_4wave_2D), 1 = the tile kernels with a
 * sweep mask, 2 = pencils with marching columns for the y-sweep, 3 =
 * pencils with warp windows for both sweeps.  All are bit-identical with
 * -fmad=false.  Returns the previous setting. */
int gclaw_split_kernel(int which);

/* y[i] = 1 / x[i] with the reciprocal the product build uses for FP64
 * divisions (a Newton-Raphson iteration from an FP32 seed; IEEE division
 * for non-positive, denormal, infinite, NaN and very large x), n device
 * values, asynchronous on stream -- exposed so its error can be measured.
 * libgclaw_strict.so, which divides exactly, exports it too. */
int gclaw_rcp_fp64(const double *x_dev, double *y_dev, long long n, void *stream);

/* Drop-in for classic2.step2 (upstream pyclaw/src/pyclaw/classic/step2.f90):
 * one unsplit step of a ghost-filled qbc.  qold_dev and qnew_dev are
 * (num_eqn, mx+4, my+4) Fortran order; the interior of qnew_dev receives the
 * updated state (its ghost entries are left untouched).  ws_dev is a
 * gclaw_ctrl used as reduction scratch (its smax_bits/blocks_done/flags must
 * be zero before the first call, which gclaw_ctrl_init ensures; each call
 * leaves them zero).  The Courant number is written to *cfl_out after the
 * stream is synchronised.  Returns GCLAW_NONPHYSICAL if a Riemann problem
 * met a non-physical state. */
int gclaw_step2(const gclaw_solver *s, const double *qold_dev, double *qnew_dev, double dt,
                gclaw_ctrl *ws_dev, double *cfl_out, void *stream);

/* Fused step with on-device boundary conditions: reads q_dev
 * (num_eqn, mx, my), applies solver.bc_lower/bc_upper as PyClaw's
 * _apply_bcs would, writes qnew_dev, and leaves the Courant number in
 * ws_dev->cfl (no synchronisation).  Replaces the pair
 * ClawSolver2D._apply_bcs + classic2.step2. */
int gclaw_step(const gclaw_solver *s, const double *q_dev, double *qnew_dev, double dt,
               gclaw_ctrl *ws_dev, void *stream);

/* Enqueue nlaunch controlled steps on stream without synchronising: each
 * reads dt and parity from ctrl_dev, steps q{parity} into q{1-parity}, and
 * its last block applies the evolve_to_time rules.  Steps after ctrl->done
 * is set return at once.  The launches can be captured in a CUDA graph. */
int gclaw_advance(const gclaw_solver *s, double *q0_dev, double *q1_dev, gclaw_ctrl *ctrl_dev,
                  int nlaunch, void *stream);

/* Dimensionally split step (Godunov splitting), the path of
 * ClawSolver2D.step() with dimensional_split=True (upstream
 * pyclaw/src/pyclaw/classic/solver.py calling classic2.step2ds with ixy=1,
 * then with ixy=2 after re-applying the boundary conditions): the x-sweep
 * of q_dev into qtmp_dev, then the y-sweep of qtmp_dev, with boundary
 * conditions applied to each input, into qnew_dev; no transverse waves.
 * The Courant number, the max of both sweeps', is left in ws_dev->cfl.
 * The three arrays are (num_eqn, mx, my), distinct, and start on a 16-byte
 * boundary (as cudaMalloc returns them; others are refused with
 * GCLAW_ERR_ARG).  Each sweep is one kernel over independent 1D problems
 * (gclaw_split_kernel). */
int gclaw_step_split(const gclaw_solver *s, const double *q_dev, double *qnew_dev,
                     double *qtmp_dev, double dt, gclaw_ctrl *ws_dev, void *stream);

/* gclaw_advance with dimensionally split steps: each of the nsteps steps is
 * two launches (x-sweep into qtmp_dev, y-sweep into the other state
 * buffer); the evolve_to_time rules apply to the whole step, so a rejected
 * step leaves q{parity} unchanged. */
int gclaw_advance_split(const gclaw_solver *s, double *q0_dev, double *q1_dev, double *qtmp_dev,
                        gclaw_ctrl *ctrl_dev, int nsteps, void *stream);

/* Device bytes gclaw_step_host needs in ws_dev. */
size_t gclaw_step_workspace_bytes(const gclaw_solver *s);

/* One step from host memory: the per-step path of the reference, where
 * ClawSolver2D.step() hands numpy arrays to classic2.step2 every step
 * (upstream pyclaw/src/pyclaw/classic/solver.py), here replacing
 * _apply_bcs + step2.  Copies q_host (num_eqn, mx, my) to the device, runs
 * gclaw_step, copies the new state to qnew_host and the Courant number to
 * *cfl_out, then synchronises the stream.  Pinned host arrays
 * (cudaHostAlloc / cudaHostRegister, e.g. torch pin_memory) are read and
 * written by the step kernel itself over NVLink-C2C, without staging
 * copies; other host memory is copied, and FP64 tile steps of grids of at
 * least eight tile rows without a periodic y boundary then run band by
 * band, the row copies on an internal stream overlapping the bands.  The
 * result is the same bits either way.  ws_dev (caller-owned, 256-byte
 * aligned, at least gclaw_step_workspace_bytes, any contents) holds the
 * control block, which each call clears, and both device states. */
int gclaw_step_host(const gclaw_solver *s, const double *q_host, double *qnew_host, double dt,
                    void *ws_dev, size_t ws_bytes, double *cfl_out, void *stream);

/* Device bytes gclaw_evolve_host needs in ws_dev. */
size_t gclaw_evolve_workspace_bytes(const gclaw_solver *s);

/* End-to-end run from host memory, the analogue of PyClaw's
 * solver.evolve_to_time: copies q_host (num_eqn, mx, my) to the device,
 * advances from t to t_end (or for max_accepted accepted steps when
 * max_accepted >= 0) with the evolve_to_time rules on the device, and copies
 * the accepted state back to q_out_host.  ws_dev (caller-owned, at least
 * gclaw_evolve_workspace_bytes) holds the two state buffers and the control
 * block; *ctrl_out receives the final control block.  Launches steps in
 * batches of `batch` (<= 0: 32) between checks of ctrl->done. */
int gclaw_evolve_host(const gclaw_solver *s, const double *q_host, double *q_out_host, double t,
                      double dt, double t_end, int max_accepted, double cfl_max,
                      double cfl_desired, double dt_max, int max_steps, void *ws_dev,
                      size_t ws_bytes, int batch, gclaw_ctrl *ctrl_out, void *stream);

/* ---- batches of independent problems ------------------------------------
 * Many problems of uneven grid sizes that share one gclaw_solver (its rp,
 * boundary conditions, limiters, order, transverse_waves, precision and
 * problem_data; its mx, my, dx, dy are ignored) advance together: each
 * launch is one attempted step of every unfinished problem, with per-problem
 * dt, CFL, rejection and stop (PyClaw's evolve_to_time rules per problem).
 * There is no reference counterpart in one call; PyClaw users loop over
 * solvers.  States of all problems live in two caller-owned FP64 buffers,
 * problem p at q_offset[p] (in doubles), each in the single-problem layout. */
typedef struct gclaw_batch_problem {
    int mx, my;          /* interior cells, >= 2 */
    double dx, dy;       /* cell sizes */
    long long q_offset;  /* offset of the problem's state in the buffers (doubles) */
} gclaw_batch_problem;

/* Device bytes of the work table for nprob problems (per problem its tile
 * and its strip decomposition, and the running starts of both). */
size_t gclaw_batch_table_bytes(int nprob);

/* Fill the work table (caller-owned device memory, 16-byte aligned) for the
 * problems described in host memory; returns the total number of tiles in
 * *total_tiles (the strip decomposition's size is kept in the table).
 * Synchronises the stream. */
int gclaw_batch_prepare(const gclaw_solver *s, const gclaw_batch_problem *probs, int nprob,
                        void *table_dev, size_t table_bytes, int *total_tiles, void *stream);

/* Initialise nprob control blocks (an array of gclaw_ctrl in device memory);
 * dt0_dev[p] is problem p's first dt (device array of nprob doubles). */
int gclaw_batch_ctrl_init(gclaw_ctrl *ctrls_dev, int nprob, const double *dt0_dev, double t,
                          double t_end, double cfl_max, double cfl_desired, double dt_max,
                          int max_steps, int max_accepted, int dt_variable, void *stream);

/* Enqueue nlaunch batched steps (no synchronisation; capturable in a CUDA
 * graph).  Each launch is a persistent grid striding over all work units of
 * all problems: tiles in FP64 (the tile body of gclaw_step), strips in
 * FP32-bulk (the strip body, or tiles while gclaw_fp32_kernel(1) is in
 * effect), so every problem evolves exactly as it would alone; problem p's
 * accepted state is in q0 or q1 per ctrls_dev[p].parity. */
int gclaw_batch_advance(const gclaw_solver *s, const void *table_dev, int nprob, int total_tiles,
                        double *q0_dev, double *q1_dev, gclaw_ctrl *ctrls_dev, int nlaunch,
                        void *stream);

/* Adjoint (reverse mode) of one step at fixed dt: lam_old = J^T lam_new with
 * J = d step(q) / d q at q = q_dev, for gradients through time stepping
 * (the reference has no adjoint).  Supported: GCLAW_RP_ACOUSTICS_2D and
 * GCLAW_RP_SHALLOW_ROE_WITH_EFIX_2D, FP64 or FP32-bulk arithmetic, lam in
 * FP64 with the layout of q.  The limiter, entropy-fix and transverse
 * min/max branches are those the forward step takes on q_dev.  lam_old_dev
 * must not alias lam_new_dev; it is overwritten.  No synchronisation. */
int gclaw_adjoint_step(const gclaw_solver *s, const double *q_dev, const double *lam_new_dev,
                       double *lam_old_dev, double dt, void *stream);

/* Allocation-free variant of gclaw_step2 (no counterpart in the reference,
 * whose Fortran step needs no device memory).  For callers that cannot
 * allocate device memory or hand over a workspace -- a Fortran/C host code
 * holding only the state arrays it was given, or a process whose device
 * memory belongs to another framework's caching allocator.  Same arguments
 * and results as gclaw_step2 minus ws_dev: the reduction scratch is a
 * file-scope __device__ array of 2 MiB + 256 B that every GPU loading the
 * library keeps until the process exits, with one slot per thread block, so
 * grids needing more than GCLAW_NOALLOC_MAX_BLOCKS thread blocks (32x8 cells
 * each in FP64, 32x16 in FP32-bulk; e.g. 33.5 M cells in FP64) are rejected
 * with GCLAW_ERR_TOO_LARGE before any launch.  The call allocates nothing
 * (no cudaMalloc/cudaFree); it clears the scratch header on the stream,
 * launches, reads the Courant number back and synchronises the stream.  The
 * first call on a device looks the scratch's device address up with
 * cudaGetSymbolAddress, so make that call before any stream capture.  All
 * calls share the one array: calls that overlap on the GPU (other streams,
 * other host threads) race and must not be issued. */
#define GCLAW_NOALLOC_MAX_BLOCKS 131072
int gclaw_step2_noalloc(const gclaw_solver *s, const double *qold_dev, double *qnew_dev,
                        double dt, double *cfl_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GCLAW_H */
