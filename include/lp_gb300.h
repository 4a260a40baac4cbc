/*
 * lp_gb300.h -- C ABI of the GB300 (sm_103a) collision/advection hot path of
 * the Landau-Poisson solver.
 *
 * Plain pointers and sizes only; every call returns an lp_status.  A context
 * owns its device buffers, its CUDA stream and its precomputed tables; it is
 * bound to the device that was current when it was created.  Contexts are not
 * thread-safe: use one context per host thread.
 *
 * Data layout (identical to the reference):
 *   state U: ncell * nv^3 records of 7 doubles (AoS),
 *            record k = s*nv^3 + (j1*nv + j2)*nv + j3, s = i1*nx2 + i2;
 *            slots 0: 1, 1: (x1-x_i1)/dx, 2: (x2-x_i2)/dx, 3..5: (v_d-v_jd)/dv,
 *            6: sum_d ((v_d-v_jd)/dv)^2.
 *   spectral arrays: n^3 complex doubles (re, im interleaved), index
 *            k + n*(j + n*i) as FFTW's row-major N x N x N.
 *   Poisson: 3 coefficients per spatial cell (mean, x-slope, y-slope).
 *
 * Reference interfaces replaced (paths relative to the reference checkout):
 *   lp_compute_q         ComputeQ      source/collisionRoutines_1.h:47
 *   lp_conserve          conserveAllMoments source/conservationRoutines.h:31
 *   lp_fft3d / lp_fs     fft3D / FS    source/collisionRoutines_1.h:40,44
 *   lp_rk4_cell          RK4           source/collisionRoutines_1.h:62
 *   lp_nodes             setInit_spectral source/SetInit_1.h:44
 *   lp_weights_rows      generate_conv_weights source/collisionRoutines_1.h:36
 *   lp_conservation_rows createCCtAndPivot source/conservationRoutines.h:34
 *   lp_poisson           pois2d        source/PoissonFunctions.h:35
 *   lp_advect_step       RK3           source/advection_1.h:70
 *   lp_collision_step    the per-cell ComputeQ/conserveAllMoments/RK4 loop and
 *                        the dU scatter of main, source/LP_ompi_1.cpp:500-568
 *   lp_step              one pass of the time loop, source/LP_ompi_1.cpp:496-621
 *   lp_set_init          SetInit_LD    source/SetInit_1.h:37
 *   lp_moments           computeMass/computeMomentum/computeKiE/computeEleE
 *                        source/MomentCalculations.h
 */
#ifndef LP_GB300_H
#define LP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    LP_OK = 0,
    LP_ERR_INVALID = 1,     /* bad argument or unsupported size */
    LP_ERR_CUDA = 2,        /* a CUDA call failed; see lp_last_error */
    LP_ERR_ALLOC = 3,       /* device or host allocation failed */
    LP_ERR_NO_DEVICE = 4,   /* no CUDA device, or not an sm_103 device */
    LP_ERR_STATE = 5        /* call out of order (e.g. no state uploaded) */
} lp_status;

/* Fixes of reference defects; LP_FIX_DEFAULT is F1 | F2 | F3 | F11 | F12. */
#define LP_FIX_F1 1u   /* RK4 reads the stride-7 slots {0,3,4,5,6} of each record */
#define LP_FIX_F2 2u   /* node sampling uses slot 3 as the v1 slope */
#define LP_FIX_F3 4u   /* collide every spatial cell (the reference: s < nx1 only) */
#define LP_FIX_F11 8u  /* snap the middle Fourier node eta[n/2] to exactly 0 */
#define LP_FIX_F12 16u /* the DG flux takes the cell integrals of E_x (dx times the
                          cell averages that pois2d leaves in IE_X, IXE_X, IXXE_X;
                          without it the electric force is 1/dx too strong) */
#define LP_FIX_DEFAULT (LP_FIX_F1 | LP_FIX_F2 | LP_FIX_F3 | LP_FIX_F11 | LP_FIX_F12)

/* Arithmetic of the collision operator. */
#define LP_PREC_FP64 0   /* every kernel in FP64 (the plain path) */
#define LP_PREC_MIXED 1  /* FP32 transforms, weight contraction and projection,
                            FP64 moments, 5x5 conservation solve and Poisson */

typedef struct {
    int nx1, nx2;     /* spatial cells along x1 and x2 (nx2 = nx1: the reference's
                         2-D grid; nx2 = 1: the 1-D reduction) */
    int nv;           /* DG velocity cells per dimension */
    int n;            /* spectral nodes per dimension (even, <= 32) */
    double lv;        /* velocity box [-lv, lv]^3, also the collision box L_v = R_v */
    double lx;        /* x1 (and x2) length */
    double nu, dt;    /* collision frequency and time step */
    double a_amp, k_wave; /* initial perturbation (1 + a cos(k x1)) */
    unsigned fixes;   /* LP_FIX_* bits */
    int precision;    /* LP_PREC_* */
    int linear_ei;    /* 1: add the linear electron-ion operator of the reference's
                         two-species variant (its FullandLinear switch,
                         collisionRoutines_1.cpp:551-737, conservationRoutines.cpp:63-98) */
} lp_params;

typedef struct lp_ctx lp_ctx;

/* ---- lifetime ---------------------------------------------------------- */
lp_status lp_ctx_create(const lp_params *p, lp_ctx **out);
lp_status lp_ctx_destroy(lp_ctx *ctx);
/* Run subsequent work on this cudaStream_t (NULL: the context's own stream). */
lp_status lp_set_stream(lp_ctx *ctx, void *cuda_stream);
lp_status lp_synchronize(lp_ctx *ctx);
/* Last error message of this context (never NULL). */
const char *lp_last_error(const lp_ctx *ctx);
/* Device bytes held by the context. */
size_t lp_device_bytes(const lp_ctx *ctx);

/* ---- state ------------------------------------------------------------- */
/* Copy the host state (n = ncell*nv^3*7 doubles) to the device and back. */
lp_status lp_set_state(lp_ctx *ctx, const double *U_host, size_t n);
lp_status lp_get_state(lp_ctx *ctx, double *U_host, size_t n);
/* Device pointer of the resident state (ncell*nv^3*7 doubles). */
lp_status lp_state_device_ptr(lp_ctx *ctx, double **U_dev);
/* Initial condition: kind 0 = the reference's Landau-damping IC (Maxwellian
 * of temperature 0.9), 1 = unit Maxwellian, 2 = two-stream with drift u. */
lp_status lp_set_init(lp_ctx *ctx, int kind, double u);

/* ---- reference-shaped routines (host pointers, one spatial cell) ------- */
lp_status lp_fft3d(lp_ctx *ctx, const double *in, double *out);
lp_status lp_fs(lp_ctx *ctx, const double *in, double *out);
lp_status lp_compute_q(lp_ctx *ctx, const double *f, double *qhat);
/* Two-species contexts (linear_ei = 1): ComputeQ's qHat (Q(f,f) plus the
 * linear term) and qHat_linear (the linear term alone), conserveAllMoments
 * of both (5 and 2 constraints), and RK4 from the conserved pair. */
lp_status lp_compute_q_lin(lp_ctx *ctx, const double *f, double *qhat, double *qhat_lin);
lp_status lp_conserve_lin(lp_ctx *ctx, double *qhat, double *qhat_lin);
lp_status lp_rk4_cell_lin(lp_ctx *ctx, const double *f, int cell, const double *qhat, const double *qhat_lin,
                          double *dU);
lp_status lp_conserve(lp_ctx *ctx, double *qhat);
/* RK4 of spatial cell `cell` from node values f and conserved qhat, reading
 * that cell's records of the resident state; dU receives nv^3*5 doubles. */
lp_status lp_rk4_cell(lp_ctx *ctx, const double *f, int cell, const double *qhat, double *dU);
/* Node values of every collided spatial cell from the resident state:
 * f receives ncell*n^3 doubles. */
lp_status lp_nodes(lp_ctx *ctx, double *f);
/* Rows [r0, r1) of the n^3 x n^3 Landau weight table gHat3(eta_xi, eta_omega). */
lp_status lp_weights_rows(lp_ctx *ctx, int r0, int r1, double *out);
/* Constraint rows C1, C2 (5 x n^3 each) and the inverse Gram matrix (5x5). */
lp_status lp_conservation_rows(lp_ctx *ctx, double *c1, double *c2, double *cct_inv);

/* ---- batched device paths (resident state) ----------------------------- */
/* Poisson solve on the resident state; potc, phix, phiy (3*ncell doubles
 * each) and fields (14*ncell: IE_X, IXE_X, IYE_X, IXXE_X, IXYE_X, IYYE_X,
 * the same six for Y, SE_X, SE_Y) are optional host outputs. */
lp_status lp_poisson(lp_ctx *ctx, double *potc, double *phix, double *phiy, double *fields);
/* Results of the last Poisson solve on the device (after lp_advect_step:
 * the solve on the third stage's input, as the reference's RK3 leaves them);
 * same outputs as lp_poisson, all optional. */
lp_status lp_last_fields(lp_ctx *ctx, double *potc, double *phix, double *phiy, double *fields);
/* One SSP-RK3 advection step of the resident state. */
lp_status lp_advect_step(lp_ctx *ctx);
/* Collision step of spatial cells [cell_begin, cell_end) of the resident
 * state (-1, -1: every collided cell). */
lp_status lp_collision_step(lp_ctx *ctx, int cell_begin, int cell_end);
/* The collision step of every collided cell with the state in HOST memory,
 * for a caller whose state lives on the host (it replaces the loop of main
 * with its scatter into U, LP_ompi_1.cpp:500-568): U_in (ncell*nv^3*7
 * doubles) is copied to the device, collided and copied back into U_out
 * (which may equal U_in).  The cells go in `chunks` (1..16) groups: the copy
 * in of one group, the collision of the previous one and the copy out of the
 * one before run at the same time (two copy streams and the context's
 * stream, joined by events), which pays once a group is still a large batch
 * (the two-stream workload's 256 cells in 4 chunks).  Successive calls
 * alternate between two device staging states, so the copy in of a call
 * overlaps the collision of the one before; with LP_HOST_ASYNC in `flags`
 * the context's stream does not wait for this call's copy out either, so
 * the next call's collision overlaps it too.  U_out is complete after
 * lp_synchronize (or, without LP_HOST_ASYNC, once the context's stream has
 * reached this call's end), and U_in must not change before then; pinned
 * (page-locked) host buffers make the copies asynchronous.  The resident
 * state (lp_set_state) is not used or changed.  More than one chunk needs
 * LP_FIX_F1 (collisions in passes of cells). */
#define LP_HOST_ASYNC 1
lp_status lp_collision_step_host(lp_ctx *ctx, const double *U_in, double *U_out, int chunks, int flags);
/* Kernel launches in one replay of the captured collision step over every
 * collided cell (its graph's kernel nodes); 0 before the first such step. */
lp_status lp_collision_graph_kernels(lp_ctx *ctx, int *kernels);
/* Programmatic kernel-to-kernel edges of that graph; 0 before the first
 * such step and by default.  With LP_PDL=1 (or 2) in the environment at
 * capture, the step graphs (collision step, time step, host-buffer collision
 * chunks, batch step) are instantiated with every edge from one kernel to the
 * next made a programmatic dependency: the next grid may be launched once
 * every block of the previous one has exited (or, with 2, started).  Each
 * kernel waits on the device for its predecessors' completion before it
 * reads anything, so results are unchanged either way. */
lp_status lp_collision_graph_edges(lp_ctx *ctx, int *programmatic);
/* nsteps passes of the time loop (advection, then collisions when nu > 0),
 * replayed from one captured CUDA graph per step. */
lp_status lp_step(lp_ctx *ctx, int nsteps);
/* out = {mass, p1, p2, p3, kinetic energy, electric energy of the last
 * Poisson solve}. */
lp_status lp_moments(lp_ctx *ctx, double *out6);

/* ---- schedule autotuner (no reference counterpart) ----------------------- */
/* A collision schedule is (cells per pass, contraction form).  The mixed
 * path has two forms of ComputeQ's weighted sum for n in {8, 16, 24, 32}:
 * line_warps 2 or 4 -- the line-tiled weighted sum with that many warps per
 * block -- and line_warps 0 -- the convolution form (the weight split into
 * seven omega factors, 3n/2-point DFTs along two axes and a direct sum along
 * the third).  The FP64 path has one form (line_warps 2). */

/* Times one collision step of the resident state (best of `reps` after a
 * warm-up, CUDA events, the state restored before each run) for every
 * candidate schedule -- cells per pass 64, 128, ... up to the workspace's
 * capacity, times the contraction forms above, the convolution form in both
 * kernel forms of lp_set_convolution_form -- and keeps the fastest; with
 * cache_path, a schedule recorded there for the same key (n, nv, lv, cells,
 * precision, device) is reused and new ones appended.  The chosen schedule
 * is returned in pass_cells and line_warps (optional); the kernel form it
 * picked is the context's convolution form afterwards
 * (lp_get_convolution_form).  Leaves the state as it was. */
lp_status lp_autotune(lp_ctx *ctx, int reps, const char *cache_path, int *pass_cells, int *line_warps);

/* Sets the schedule directly: pass_cells a multiple of 32 up to the
 * workspace capacity (lp_autotune's largest candidate), line_warps one of
 * the forms above.  LP_ERR_INVALID for a schedule the context cannot run. */
lp_status lp_set_schedule(lp_ctx *ctx, int pass_cells, int line_warps);

/* The kernels of the convolution form (mixed path, line_warps 0): form 1
 * (default) keeps the axis-2 spectra on chip -- the axis-3 DFTs go to
 * device memory, then one kernel per (k3, group of cells) runs the axis-2
 * DFTs, the direct sums along axis 1 and the inverse axis-2 DFTs, its
 * operands brought in by bulk copies -- form 0 runs the axis-3/axis-2 DFTs,
 * the axis-1 sums and the inverse axis-2 DFTs as three kernels through
 * device memory.  Both forms agree to FP32 rounding.  The environment
 * variable LP_FQ_FUSED=0 makes form 0 the default of new contexts; the
 * autotuners time both and keep the faster (form 1 at n <= 24, form 0 at
 * n = 32 on GB300).  A pass runs the convolution in chunks of cells, 64 or
 * more while their scratch stays within 512 MB; LP_FQ_CHUNK=<cells> (a
 * multiple of 32) in the environment at context creation sets a smaller
 * chunk.  The chunk changes no result: each cell's sums are the same. */
lp_status lp_set_convolution_form(lp_ctx *ctx, int form);
lp_status lp_get_convolution_form(const lp_ctx *ctx, int *form);

/* ---- measurement helpers (no reference counterpart) --------------------- */
/* Average device time in ms of one launch of a hot-path stage on the
 * context's stream, over `reps` launches after one warm-up, timed with CUDA
 * events: which = 0 the weighted contraction of ComputeQ for every collided
 * cell, 1 the forward transform, 2 the moment-conserving projection, 3 the
 * DG projection of the RK4 combination; 4, 6, 7, 8 the kernels of the
 * convolution form for the first convolution chunk of cells, each alone,
 * when that form is the schedule: form 1 -- 4 the axis-3 DFTs, 6 the fused
 * axis-2 DFTs / axis-1 sums / inverse axis-2 DFTs, 8 the inverse axis-3
 * DFTs (5 and 7 launch nothing); form 0 -- 4 the axis-3 and axis-2 DFTs in
 * one kernel, 6 the axis-1 sums, 7 the inverse axis-2 DFTs, 8 the inverse
 * axis-3 DFTs (5 launches nothing).  Needs the resident state. */
lp_status lp_time_kernel(lp_ctx *ctx, int which, int reps, double *ms);
/* Dense FMA throughput of the current device measured with dependent-chain
 * microbenchmarks: FP32 (packed f32x2) and FP64, in TFLOP/s. */
lp_status lp_measure_fp_peaks(double *fp32_tflops, double *fp64_tflops);

/* ---- diagnostics and state I/O ------------------------------------------ */
/* The reference's per-step diagnostics of the resident state, computed on the
 * device after a Poisson solve of that state (LP_ompi_1.cpp:452-470):
 * out10 = {mass, p1, p2, p3, kinetic energy, electric energy EE, sqrt(EE),
 * log sqrt(EE), total energy, entropy int f log f} (computeMass,
 * computeMomentum, computeKiE, computeEleE in MomentCalculations.cpp,
 * computeEntropy in EntropyCalculations.cpp:11-65; the entropy's integrand is
 * evaluated in FP32). */
lp_status lp_diagnostics(lp_ctx *ctx, double *out10);
/* Appends the reference's moment line (9 values, "%11.8g") to moments_path
 * and its entropy line (entropy, log|entropy|, log|log|entropy||) to
 * entropy_path; either may be NULL. */
lp_status lp_diagnostics_append(lp_ctx *ctx, const char *moments_path, const char *entropy_path);
/* The reference's (x1, v1) marginal (PrintMarginal, MarginalCreation.cpp:174)
 * at 4 x 4 points per (x1 cell, v1 cell): out[nx1*4][nv*4]. */
lp_status lp_marginal_x1v1(lp_ctx *ctx, double *out);
/* Snapshot files in the reference's format (LP_ompi_1.cpp:416-438, 628): raw
 * native-endian doubles of the state, snapshots appended one after another;
 * restart reads the last snapshot and rejects a file whose size is not a
 * whole number of states. */
lp_status lp_state_append(lp_ctx *ctx, const char *path);
lp_status lp_state_restart(lp_ctx *ctx, const char *path);

/* ---- adjoint ------------------------------------------------------------- */
/* No counterpart in the reference.  Hand-written vector-Jacobian products of
 * the FP64 path (contexts with LP_PREC_FP64 and LP_FIX_F1 | LP_FIX_F2 |
 * LP_FIX_F3; Poisson matrix of order 3*nx1*nx2 <= 4096), evaluated at the
 * resident state, which they leave unchanged.  Adjoint vectors are DEVICE
 * pointers of ncell*nv^3*7 doubles in the state's layout.
 *   collision step: the bilinear ComputeQ linearised (correlations of the
 *     adjoint with the convolution form's arrays, lp_set_adjoint_form), the
 *     transposed transforms, the self-adjoint conservation
 *     projection and the transposed DG projection, through the RK4 stages;
 *   advection step: the transposed upwind DG flux of each SSP-RK3 stage and
 *     the transposed LDG Poisson solve of its field;
 *   field energy J = 1/2 sum_cells dx dy (E_0^2 + (E_1^2 + E_2^2)/12) over E_x
 *     and E_y of the Poisson solve on the state. */
/* The form of ComputeQ's VJP in the collision step's adjoint: 0 (default)
 * the two families of correlations of lam_q with the omega-factor arrays of
 * the convolution form, by 3n/2-point DFTs along the three axes; 1 the
 * gather over the pair table of the weighted sum.  Both give the transpose of
 * source/collisionRoutines_1.cpp:739-822 linearised at F. */
lp_status lp_set_adjoint_form(lp_ctx *ctx, int form);
/* J of the resident state and, when lam_U_dev is not NULL, dJ/dU. */
lp_status lp_field_energy(lp_ctx *ctx, double *J, double *lam_U_dev);
/* lam_in = (d collision step / dU)^T lam_out; *dJ_dnu (optional) = the
 * derivative of <lam_out, step output> with respect to nu. */
lp_status lp_collision_vjp(lp_ctx *ctx, const double *lam_out_dev, double *lam_in_dev, double *dJ_dnu);
/* lam_in = (d advection step / dU)^T lam_out. */
lp_status lp_advect_vjp(lp_ctx *ctx, const double *lam_out_dev, double *lam_in_dev);
/* The same for one whole time step (advection, then collisions). */
lp_status lp_step_vjp(lp_ctx *ctx, const double *lam_out_dev, double *lam_in_dev, double *dJ_dnu);
/* Gradient of the field energy after nsteps time steps from the resident
 * (initial) state: J, dJ/dU0 (device) and dJ/dnu, by the adjoint with a
 * checkpoint every `checkpoint` steps (the states between checkpoints are
 * recomputed segment by segment). */
lp_status lp_field_energy_gradient(lp_ctx *ctx, int nsteps, int checkpoint, double *J, double *dJ_dU0_dev,
                                   double *dJ_dnu);

/* ---- batches of independent runs ---------------------------------------- */
/* No counterpart in the reference, which runs one instance per job.  A batch
 * steps `count` independent runs, each with its own lp_params (grid nx1 x nx2,
 * nv, n, lv, lx, nu, dt, initial-condition parameters); fixes and precision
 * must agree across runs and include LP_FIX_F1 (collisions run in passes of
 * cells), and 2-D runs need LP_FIX_F3.  Runs with equal (n, nv, lv) form a
 * class: their spatial cells go through one set of collision launches with
 * per-cell nu and dt, over one shared weight table.  Every run is advected on
 * its own stream and every class collided on its own stream; lp_batch_step
 * replays one captured CUDA graph per time step.  A run whose nu is 0 still
 * passes through its class's collision launches (an increment of zero). */
typedef struct lp_batch lp_batch;
lp_status lp_batch_create(const lp_params *params, int count, lp_batch **out);
lp_status lp_batch_destroy(lp_batch *b);
lp_status lp_batch_set_stream(lp_batch *b, void *cuda_stream);
lp_status lp_batch_synchronize(lp_batch *b);
const char *lp_batch_last_error(const lp_batch *b);
size_t lp_batch_device_bytes(const lp_batch *b);
/* State of run `run` (its nx1*nx2*nv^3*7 doubles), as lp_set_state etc. */
lp_status lp_batch_set_state(lp_batch *b, int run, const double *U_host, size_t n);
lp_status lp_batch_get_state(lp_batch *b, int run, double *U_host, size_t n);
lp_status lp_batch_set_init(lp_batch *b, int run, int kind, double u);
lp_status lp_batch_moments(lp_batch *b, int run, double *out6);
lp_status lp_batch_advect_step(lp_batch *b);
lp_status lp_batch_collision_step(lp_batch *b);
lp_status lp_batch_step(lp_batch *b, int nsteps);
/* Classes and their schedules: info6 = {n, nv, runs, cells, cells per pass,
 * warps per line block}; tuned_ms (optional) = the class's collision step
 * time measured by the autotuner (0 if not tuned). */
int lp_batch_classes(const lp_batch *b);
lp_status lp_batch_class_info(const lp_batch *b, int cls, int *info6, double *tuned_ms);
/* Autotuner: for every class, time one collision step (best of `reps` after
 * a warm-up, CUDA events, the class state restored before each run) for
 * every candidate schedule -- cells per pass 64, 128, ... up to the
 * workspace's capacity; 2 or 4 warps per block of the line-tiled
 * contraction, or the convolution form in either kernel form -- and keep
 * the fastest.  With cache_path, schedules already
 * recorded there for the same key (n, nv, lv, cells, precision, device) are
 * reused and new ones appended.  Needs every run's state; leaves it as it
 * was. */
lp_status lp_batch_autotune(lp_batch *b, int reps, const char *cache_path);

/* ---- x1 slabs of a sharded run ------------------------------------------ */
/* Replace the reference's MPI decomposition (cells split over ranks,
 * source/LP_ompi_1.cpp:164-178; the whole state root-gathered and broadcast
 * every step, LP_ompi_1.cpp:518-567, and in RK3, advection_1.cpp:472-489) by
 * contiguous x1 slabs.  A slab context holds global x1 rows [i1_begin,
 * i1_end) of the grid `global` as its local rows 1..i1_end-i1_begin, plus one
 * halo row on each side (local rows 0 and i1_end-i1_begin+1; its state has
 * (i1_end-i1_begin+2)*nx2*nv^3 records).  One time step on the slab is, for
 * stage = 0, 1, 2 of SSP-RK3:
 *   1. the caller copies the neighbour slabs' edge rows of stage buffer
 *      `stage` into its halo rows (periodic in x1);
 *   2. lp_slab_charge: the charge moments of the own cells of that buffer;
 *   3. the caller all-gathers them in x1 order (3 per cell, global order);
 *   4. lp_slab_fields: the global LDG Poisson solve from them (every rank
 *      solves the same small system) and the field integrals of its rows;
 *   5. lp_slab_advect_stage: the stage's flux and update of every record;
 * then lp_collision_step over the own cells (cells nx2 .. (i1_end-i1_begin+1)
 * *nx2), which needs no exchange.  The advection of a slab runs in FP64 for
 * either precision.  lp_set_init places the slab in the global grid. */
lp_status lp_slab_create(const lp_params *global, int i1_begin, int i1_end, lp_ctx **out);
/* Device pointer of stage buffer `stage` of the state: 0 = U (the step's
 * input and, after stage 2, its output), 1 = U1, 2 = Ut (the inputs of
 * stages 1 and 2), records in the state's layout. */
lp_status lp_stage_device_ptr(lp_ctx *ctx, int stage, double **dev);
/* Charge moments (3 per cell, the reference's order and sums) of the own
 * cells of stage buffer `stage` into rt_dev (device, 3*(i1_end-i1_begin)*nx2
 * doubles). */
lp_status lp_slab_charge(lp_ctx *ctx, int stage, double *rt_dev);
/* LDG Poisson solve of the whole grid from its charge moments rt_global_dev
 * (device, 3*nx1*nx2 doubles in global cell order), and the field integrals
 * of the slab's rows (halo rows included) for the next lp_slab_advect_stage. */
lp_status lp_slab_fields(lp_ctx *ctx, const double *rt_global_dev);
/* SSP-RK3 stage `stage` (0, 1, 2) of every record of the slab with the field
 * integrals of the last lp_slab_fields (FP64). */
lp_status lp_slab_advect_stage(lp_ctx *ctx, int stage);
/* Potential and field coefficients of the whole grid from the last
 * lp_slab_fields (host, 3*nx1*nx2 doubles each; any may be NULL). */
lp_status lp_slab_fields_host(lp_ctx *ctx, double *potc, double *phix, double *phiy);

/* ---- allocation-free projection ---------------------------------------- */
/* No counterpart in the reference.  The moment-conserving projection of
 * lp_conserve for `ncell` mode arrays at once, for callers that may not
 * allocate device memory when they call it: code whose device memory belongs
 * to another framework's pool, or a time-critical loop in which cudaMalloc
 * and cudaFree (which can synchronise the whole device) are not allowed.
 * Nothing is allocated: the caller passes, in device memory it owns,
 *   qhat_dev     ncell x n3 complex doubles (re, im interleaved), the
 *                reference's layout, projected in place (16-byte aligned);
 *   c1_dev, c2_dev  the 5 x n3 constraint rows and cct_inv_dev the inverse
 *                Gram matrix (25 doubles), e.g. copied from
 *                lp_conservation_rows;
 * and the work runs on cuda_stream (NULL: the legacy default stream).
 * Scratch lives in one fixed device array inside the library sized for
 * LP_NOALLOC_MAX_CELLS cells (about 2.8 MB, held by every GPU that loads the
 * library until the process exits); larger ncell is rejected with
 * LP_ERR_INVALID.  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress) with the device current; make that first
 * call before any stream capture.  That address is kept for the life of the
 * process: do not call this function again after a cudaDeviceReset of that
 * device.  An error already pending on the calling thread is reported as
 * LP_ERR_CUDA (and left pending) before anything is launched.  All calls
 * share the array: calls whose work overlaps on the GPU race and must be
 * serialised. */
#define LP_NOALLOC_MAX_CELLS 4096
lp_status lp_conserve_noalloc(double *qhat_dev, int ncell, int n3, const double *c1_dev,
                              const double *c2_dev, const double *cct_inv_dev, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
