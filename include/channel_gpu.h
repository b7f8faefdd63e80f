/*
 * channel_gpu.h -- C ABI of the GB300 (sm_103a) RK3-substep library for the
 * staggered finite-difference channel solver of Adrian-Lozano/channel-flow.
 *
 * One context holds one channel, device-resident between calls.  Host arrays
 * crossing this boundary use the reference's Fortran layout and extents
 * (column-major, 1-based in the Fortran sense, ghosts and periodic duplicate
 * planes included):
 *     U    (nx,  ny+1, nz+1)      V (nx+1, ny, nz+1)      W (nx+1, ny+1, nz)
 *     P    (nx+1, ny+1, nz+1)     nu_t (nx+1, ny+1, nz+1)
 * where nx, ny, nz are the face counts of the input_parameters file
 * (initialization.f90:79-124).  All functions return 0 on success and a
 * nonzero CF_ERR_* code otherwise; cf_last_error() gives the message.  Calls
 * on one context must be serialised by the caller; separate contexts are
 * independent.  The reference has no return codes (it calls Stop); the
 * checks it makes with Stop are made here and reported as CF_ERR_INVALID.
 */
#ifndef CHANNEL_GPU_H
#define CHANNEL_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cf_ctx cf_ctx;

enum {
    CF_OK = 0,
    CF_ERR_INVALID = 1,   /* bad size or parameter (the reference's Stop)      */
    CF_ERR_CUDA = 2,      /* CUDA runtime error                                */
    CF_ERR_UNSUPPORTED = 3, /* model the library does not implement           */
    CF_ERR_IO = 4,        /* file read/write error                             */
    CF_ERR_NAN = 5        /* NaN found by a check                              */
};

enum { CF_PREC_FP64 = 0, CF_PREC_SPLIT = 1 };

/* Scalars read by read_input_parameters (input_output.f90:21-133), plus
 * options of this library that the reference hard-codes. */
typedef struct {
    double nu;             /* viscosity                                         */
    double CFL;            /* CFL number; CFL < 0 means dt = -CFL               */
    double dPdx, dPdz;     /* imposed pressure gradients                        */
    double Rossby_plus;    /* Omega_z = Rossby_plus*sqrt(dPdx)/2                */
    double freq_mult;      /* target centre-line velocity when x_mass_cte == 2  */
    int Retau_int;         /* mass-flow rescale flag (initialization.f90:433)   */
    int x_mass_cte;        /* 0 fixed dPdx, 1 constant mass flow, 2 centre-line */
    int y_mass_cte;        /* 1 constant mass flow in y                         */
    int LES_model;         /* 0 none, 2 dynamic Smagorinsky, 3 AMD              */
    int iwall_model;       /* 0 no-slip walls, 3 equilibrium wall model         */
    int Dirichlet_nu_t;    /* ghost rule for nu_t: 1 Dirichlet, 0 Neumann, 2 (AMD
                              only) -nu_t(2) + 0.38 dPdx^(1/2) (y(2)-y(1))       */
    int jref_eqwm;         /* eqwm matching index                               */
    /* library options (not in input_parameters) */
    int precision;         /* CF_PREC_FP64 or CF_PREC_SPLIT                     */
    int eqwm_ncv;          /* eqwm ODE cells (reference: 100, wallmodel.f90:621) */
    double eqwm_stretch;   /* eqwm ODE stretching (reference: 1.10)             */
    int sgs_recompute;     /* 1: evaluate the second eddy viscosity of substep 1
                              (time_integration.f90:103) inside cf_time_step_rk3;
                              0: reuse the first one (bit-identical inputs)      */
    int dsm_unfused;       /* 1: evaluate the dynamic Smagorinsky model with the
                              multi-pass kernels even where the fused pass applies;
                              2: the same with the filter kernel's per-element
                              plane gather instead of tensor copies             */
    int cfl_corrected;     /* 1: convective limit of compute_dt with the minimum
                              over cells of spacing/|u| (the reference takes the
                              maximum, time_integration.f90:191-201, which leaves
                              only the viscous limit and the 5e-3 cap); 0: as the
                              reference (default) */
} cf_params;

/* Fills p with the defaults of the library (reference values where the
 * reference hard-codes them). */
void cf_default_params(cf_params *p);

/* ---- lifetime --------------------------------------------------------- */
/* Replaces initialize (initialization.f90:23-536) for one slab holding the
 * whole domain.  x, y, z are host face coordinates of lengths nx, ny, nz
 * (the mesh records of the snapshot file, input_output.f90:244-254). */
int cf_create(int nx, int ny, int nz, const double *x, const double *y, const double *z,
              const cf_params *p, int device, cf_ctx **out);
int cf_destroy(cf_ctx *ctx);
/* Message of the last failure on ctx; with ctx == NULL, of the last failure
 * of this thread that had no context (e.g. cf_create). */
const char *cf_last_error(const cf_ctx *ctx);

/* ---- state transfer (host <-> device) ---------------------------------- */
/* Uploads U, V, W (the snapshot body, input_output.f90:276-362) and sets
 * Uo = U etc. (input_output.f90:380-382). */
int cf_upload_fields(cf_ctx *ctx, const double *U, const double *V, const double *W);
/* Any pointer may be NULL.  P is the pressure stored at substep 1 of the last
 * projection (projection.f90:129-137); nu_t the last eddy viscosity. */
int cf_download_fields(cf_ctx *ctx, double *U, double *V, double *W, double *P, double *nu_t);
/* Wall-model arrays: alpha_x (nx,2,nz+1), alpha_z (nx+1,2,nz),
 * tau_eqwm_initial (nx,2,nz+1).  Any pointer may be NULL. */
int cf_download_wall(cf_ctx *ctx, double *alpha_x, double *alpha_z, double *tau);
int cf_upload_wall(cf_ctx *ctx, const double *alpha_x, const double *alpha_z, const double *tau);

/* Module scalars of global.f90 the path reads or writes. */
int cf_set_scalars(cf_ctx *ctx, double t, double dt, int rk_step, double dPdx, double dPdy);
int cf_get_scalars(cf_ctx *ctx, double *t, double *dt, int *rk_step, double *dPdx, double *dPdy);

/* initialization.f90:432-463: initial mass flow Qflow_x_0 (with the Retau
 * rescale of U when Retau_int != 0).  Call after cf_upload_fields. */
int cf_init_mass_flow(cf_ctx *ctx, double *Qflow_x_0);

/* ---- mirrors of the subroutines time_integration.f90 calls ------------ */
int cf_compute_dt(cf_ctx *ctx, double *dt);                       /* time_integration.f90:179 */
int cf_compute_eddy_viscosity(cf_ctx *ctx);                       /* subgrid.f90:23           */
int cf_compute_wall_model(cf_ctx *ctx);                           /* wallmodel.f90:24         */
int cf_compute_rhs_u(cf_ctx *ctx, int slot);                      /* equations.f90:24  -> Fu{slot} */
int cf_compute_rhs_v(cf_ctx *ctx, int slot);                      /* equations.f90:186 -> Fv{slot} */
int cf_compute_rhs_w(cf_ctx *ctx, int slot);                      /* equations.f90:351 -> Fw{slot} */
int cf_rk_update(cf_ctx *ctx, int substep);                       /* time_integration.f90:108-146 */
int cf_apply_boundary_conditions(cf_ctx *ctx);                    /* boundary_conditions.f90:20 */
int cf_compute_projection_step(cf_ctx *ctx);                      /* projection.f90:20        */
int cf_compute_dPx_for_constant_mass_flow(cf_ctx *ctx, double *dPdx); /* mass_flow.f90:103  */
int cf_compute_dPy_for_constant_mass_flow(cf_ctx *ctx, double *dPdy); /* mass_flow.f90:147  */
int cf_compute_dPx_for_constant_Ucenterline(cf_ctx *ctx, double *dPdx); /* mass_flow.f90:192 */
int cf_check_divergence(cf_ctx *ctx, double *maxdiv, double *maxabsdiv); /* projection.f90:234 */
/* Actual pressure of the current fields into P: compute_pressure
 * (pressure.f90:21), which output_data calls before writing a snapshot
 * (input_output.f90:401-404).  Uses the current nu_t and avg_nu_t and the
 * Poisson matrix of the projection.  Writes P on i = 2..nxg-1, j = 1..nyg,
 * k = 2..nzg-1 (the z duplicate plane and the x duplicate column included);
 * the x ghost columns i = 1, nxg and z ghost planes k = 1, nzg keep their
 * values.  Overwrites the right-hand sides of slot 1 (with zero wall rows in
 * Fv1).  The next rk_step-1 projection replaces P with the pseudo-pressure,
 * as in the reference. */
int cf_compute_pressure(cf_ctx *ctx);
/* U(interior) += value (comp 0) or V(interior) += value (comp 1), then
 * dPdx (dPdy) = value/dt: the driver lines time_integration.f90:155-156, 168-169. */
int cf_apply_mass_flow_correction(cf_ctx *ctx, int comp, double value);
/* Save Uo = U (time_integration.f90:94-97). */
int cf_save_old_state(cf_ctx *ctx);
/* Downloads one of the RK right-hand sides Fu/Fv/Fw{slot} with the extents of
 * the matching velocity field; the interior ranges of initialization.f90:419-429
 * hold the values, the rest is unspecified. comp: 0 u, 1 v, 2 w. */
int cf_download_rhs(cf_ctx *ctx, int comp, int slot, double *out);
/* Downloads avg_nu_t (1, ny+1, 1), the plane coefficient <LM>/<MM>. */
int cf_download_avg_nu_t(cf_ctx *ctx, double *out);
/* eqwm counters of the last wall-model call (wallmodel.f90:623-653). */
int cf_get_eqwm_counters(cf_ctx *ctx, int *n_nan, int *n_iter);
/* The multi-pass dynamic Smagorinsky filter kernel of the FP32 path gathers
 * its planes with tensor copies and waits for each with a time limit (0.2 s);
 * a block whose wait expired stops and is counted.  cf_copy_wait_expired
 * synchronises, returns that count since the last query in *expired and
 * clears it; cf_compute_eddy_viscosity and cf_time_step_rk3 (sync != 0)
 * return CF_ERR_CUDA when it is nonzero.  cf_test_skip_plane_copy (a test
 * hook) leaves out the first plane copy of every block so that its wait
 * expires. */
int cf_copy_wait_expired(cf_ctx *ctx, int *expired);
int cf_test_skip_plane_copy(cf_ctx *ctx, int on);
/* The inputs the equilibrium wall model hands to its ODE solve for the
 * current fields (wallmodel.f90:597-621): *npts = nx * 2 * (nz+1) wall
 * points, u_les (device array of cap >= *npts doubles, wall-point order
 * (i, wall, k); may be NULL to query *npts) the matching-plane velocity
 * magnitude of each, *h_wm the matching height yg(jref_eqwm), *nu the
 * viscosity (either may be NULL).  iwall_model 3 only.  Used to draw the
 * learned wall stress's training samples from the solver's own runs. */
int cf_wall_model_inputs(cf_ctx *ctx, double *u_les, long cap, long *npts, double *h_wm, double *nu);

/* ---- fast path ------------------------------------------------------- */
/* compute_dt followed by compute_time_step_RK3 (time_integration.f90:89-173,
 * including the mass-flow forcing), nsteps times, fully on the device with
 * dt and dPdx kept in device memory.  Enqueued on the context's stream; the
 * call returns without waiting unless sync != 0.  The step sequence is
 * captured once into a CUDA graph and replayed. */
int cf_time_step_rk3(cf_ctx *ctx, int nsteps, int sync);
/* Same sequence with a fixed dt (the reference's CFL < 0 rule). */
int cf_set_fixed_dt(cf_ctx *ctx, double dt);
int cf_synchronize(cf_ctx *ctx);
/* The cudaStream_t the context launches on (for event timing by callers). */
void *cf_get_stream(cf_ctx *ctx);
/* Count of kernel launches one cf_time_step_rk3 step enqueues. */
int cf_launches_per_step(cf_ctx *ctx);
/* Runs nsteps steps of the fast-path sequence without the graph, timing every
 * kernel with CUDA events on the context's stream; returns per-kernel total
 * device milliseconds and launch counts (names: max_names rows of 48 chars). */
int cf_profile_steps(cf_ctx *ctx, int nsteps, int max_names, char *names, double *total_ms, int *counts,
                     int *n_names);
/* The same per-kernel figures from the graph form of the step: each of the
 * nsteps steps is captured with an event-record node after every kernel,
 * launched as one graph (as cf_time_step_rk3 replays it) and timed from those
 * events. */
int cf_profile_graph_steps(cf_ctx *ctx, int nsteps, int max_names, char *names, double *total_ms, int *counts,
                           int *n_names);

/* Empirical tuning of the z-chunk counts of the marching kernels (fused
 * right-hand side, fused dynamic Smagorinsky pass or AMD pass) on the
 * current state: every admissible count is timed (reps launches each, CUDA
 * events) and the fastest kept; the state is unchanged.  report (6 doubles,
 * may be NULL): chosen right-hand-side chunks and its microseconds, chosen
 * DSM chunk length and its microseconds, chosen AMD chunks and its
 * microseconds (0 where not tuned).  Call after at least one step. */
int cf_autotune(cf_ctx *ctx, int reps, double *report);

/* ---- statistics (statistics.f90:22-171) ------------------------------ */
/* out: 9 profiles of length ny (Umean, Vmean, Wmean, U2mean, V2mean, W2mean,
 * UVmean, Pmean, P2mean) followed by utau, Retau, Qflow_x, Qflow_y,
 * dU/dy at the bottom and top walls, and the wall averages of nu_t
 * (9*ny + 8 values). */
int cf_compute_statistics(cf_ctx *ctx, double *out);
/* The reductions of output_monitor (monitor.f90:20-52) on the current
 * fields: out[9] = mean U, V, W over the interior ranges divided by
 * (nx-1)(ny-1)(nz-1), max U, V, W, mean nu_t (interior sum divided by
 * (nx+1)(ny+1)(nz+1)), max nu_t, and check_divergence's max (signed)
 * divergence.  The printing itself is the caller's (channelflow's
 * Channel.output_monitor mirrors it). */
int cf_output_monitor(cf_ctx *ctx, double *out);

/* ---- input_parameters file and snapshot format ----------------------- */
/* Parses the reference's input_parameters text (input_output.f90:29-81).
 * grid[3] receives nx, ny, nz; files receive filein/fileout (200 chars);
 * ints[4] nsteps, nsave, nstats, nmonitor; ints2[2] nstep_init, random_init. */
int cf_read_input_parameters(const char *path, cf_params *p, int grid[3], char filein[200], char fileout[200],
                             int ints[4], int ints2[2]);
/* Snapshot in the reference's big-endian stream format
 * (input_output.f90:231-384 read, 393-544 write): mesh records for x, y, z,
 * xm, ym, zm, then U, V, W (and, on write, P and nu_t) with int32 shapes.
 * Read: x,y,z must hold nx,ny,nz doubles; U,V,W reference extents. */
int cf_read_snapshot(const char *path, int nx, int ny, int nz, double *x, double *y, double *z, double *U,
                     double *V, double *W);
int cf_write_snapshot(const char *path, int nx, int ny, int nz, const double *x, const double *y, const double *z,
                      const double *U, const double *V, const double *W, const double *P, const double *nu_t);
/* Statistics text file of output_statistics (input_output.f90:549-570):
 * a header '%', t, Retau, utau, nu (F15.8), nx, ny, nz, istep (I12), then
 * one record per face row j = 1..ny of y, Umean, U2mean, V2mean, W2mean,
 * UVmean, P2mean (F15.8).  stats is the output of cf_compute_statistics
 * (Retau and utau are taken from it); y holds ny faces. */
int cf_write_statistics(const char *path, double t, double nu, int nx, int ny, int nz, int istep, const double *y,
                        const double *stats);
/* The reference's file name for it: fileout.<istep+nstep_init>.stats.txt
 * (input_output.f90:557-558); fails when it needs more than cap bytes. */
int cf_statistics_file_name(const char *fileout, int istep, int nstep_init, char *name, int cap);

/* ---- learned wall-stress model ----------------------------------------
 * A 3 -> 64 -> 64 -> 1 tanh network standing in for the equilibrium wall
 * model's ODE solve (solve_u_eqwm, eqwm.f90:90-223, called per wall point at
 * wallmodel.f90:621): inputs log(u_les), log(matching height), log(nu),
 * output log(tau_w h / (nu u_les)) (the stress over its laminar value), all
 * normalised with the training set's mean and standard deviation.  BF16 weights, FP32 accumulation; the 64 x 64 layer of
 * the inference runs on the tensor cores.  No counterpart in the reference.
 * Device pointers throughout; every call is ordered on `stream` (NULL: the
 * legacy default stream). */
typedef struct cf_mlp cf_mlp;
enum { CF_MLP_NPARAM = 4481 };
/* eqwm solve per sample: u, h, nu (n each) -> tau (and the Picard passes,
 * may be NULL); ODE grid of ncv cells with stretching `stretch`, warm start
 * tau_init; the reference's non-convergence rule (101 passes) is reported in
 * iters, not replaced. */
int cf_eqwm_solve_batch(int n, const double *u, const double *h, const double *nu, int ncv, double stretch,
                        double tau_init, double *tau, int *iters, void *stream);
/* A network with seeded (Xavier-uniform) weights for eqwm with (ncv, stretch). */
int cf_mlp_create(int seed, int ncv, double stretch, cf_mlp **out);
int cf_mlp_destroy(cf_mlp *m);
/* Sets the normalisation and the training envelope from a training set
 * (means and standard deviations of the three input logs and the target,
 * per-input min and max of the logs). */
int cf_mlp_fit_normalisation(cf_mlp *m, int n, const double *u, const double *h, const double *nu,
                             const double *tau, void *stream);
/* Mini-batch Adam on mean((y - target)^2): `epochs` passes over n
 * samples in batches of `batch` (a multiple of 128) with a seeded
 * permutation per epoch, step size lr decayed by cosine to lr/100.
 * loss_out (epochs values, may be NULL): mean batch loss per epoch. */
int cf_mlp_train(cf_mlp *m, int n, const double *u, const double *h, const double *nu, const double *tau, int epochs,
                 int batch, double lr, int seed, double *loss_out, void *stream);
/* Gradient of the batch loss over samples 0..n-1 (n a multiple of 128) at
 * the current parameters, into grad (CF_MLP_NPARAM doubles, device). */
int cf_mlp_gradient(cf_mlp *m, int n, const double *u, const double *h, const double *nu, const double *tau,
                    double *grad, double *loss, void *stream);
/* on = 1 (default): cf_mlp_train and cf_mlp_gradient run layer 2's three
 * products (forward, input gradient, weight gradient) on the tensor cores,
 * BF16 operands with FP32 accumulation (the output gradient of layer 2
 * rounded to BF16 where it feeds them); 0: the FP32-pipe gradient kernel
 * (layer-2 output gradient in FP32). */
int cf_mlp_set_train_tensor_cores(cf_mlp *m, int on);
/* tau = network(u, h, nu); use_tensor_cores 0 runs the same arithmetic on
 * the FP32 pipes (the cross-check).  inside (may be NULL): 1 where all three
 * inputs lie within the training envelope. */
int cf_mlp_predict(cf_mlp *m, int n, const double *u, const double *h, const double *nu, double *tau, int *inside,
                   int use_tensor_cores, void *stream);
/* FP32 master parameters (CF_MLP_NPARAM floats, host) and the normalisation
 * (8 doubles: means, standard deviations) and envelope (6 doubles: min, max
 * of the three input logs). */
int cf_mlp_get(cf_mlp *m, float *params, double *norm, double *envelope);
int cf_mlp_set(cf_mlp *m, const float *params, const double *norm, const double *envelope);
/* 1 in *expired when a tensor-core inference of m since the last call gave up
 * waiting for its MMA (each wait is bounded: 1 s, then a second bounded wait
 * before the kernel frees its tensor memory); the record is then cleared.
 * Samples of the tiles not finished are marked outside the envelope, so that
 * the wall model solves eqwm for them.  Synchronises the device. */
int cf_mlp_wait_expired(cf_mlp *m, int *expired);
/* Test hook: on = 1 makes the tensor-core inference issue no MMA, so that its
 * bounded waits run out (about 2 s per launch) -- the path above is exercised
 * without faulting anything.  0 (default) restores normal inference. */
int cf_mlp_test_skip_mma(cf_mlp *m, int on);
/* Uses the network for the wall stress of ctx's equilibrium wall model
 * (iwall_model 3): points whose inputs fall outside the envelope, and all
 * points when m is NULL, keep the eqwm solve.  Every `check_every` calls of
 * the wall model (0: never) the eqwm solve also runs for all points and the
 * relative error of the network against it is recorded.  ctx's eqwm_ncv and
 * eqwm_stretch must be those m was trained for.  m must outlive its use. */
int cf_set_wall_mlp(cf_ctx *ctx, cf_mlp *m, int check_every);
/* The last check: out[5] = wall-model calls so far, max and mean
 * |tau_mlp - tau_eqwm|/tau_eqwm over the points the network served, points
 * served, points that fell back to eqwm. */
int cf_get_wall_mlp_log(cf_ctx *ctx, double *out);

/* ---- ensembles of independent channels ---------------------------------
 * Members are contexts created by cf_create (any grids and parameters, one
 * device) and stay owned by the caller.  cf_ensemble_step advances every
 * member by nsteps steps of cf_time_step_rk3; one step of the ensemble is
 * one CUDA graph with a branch per member, replayed (captured again only for
 * a new combination of the members' buffer rotations), so the members run
 * concurrently.  The ensemble's stream orders the work; the members' streams
 * are made to wait for it before the call returns.  A member must not be
 * used on its own while an ensemble step is in flight.  No counterpart in the
 * reference. */
typedef struct cf_ensemble cf_ensemble;
int cf_ensemble_create(int n, cf_ctx *const *members, cf_ensemble **out);
int cf_ensemble_destroy(cf_ensemble *e);
int cf_ensemble_step(cf_ensemble *e, int nsteps, int sync);
void *cf_ensemble_stream(cf_ensemble *e);
/* Kernel launches one ensemble step holds (all members). */
int cf_ensemble_launches_per_step(cf_ensemble *e);
/* 1 (default): the members' steps run in four segments and the tridiagonal
 * systems of all members -- every (member, kx, kz) mode -- are solved by one
 * FP64 launch between segments (split-path members then get FP64 solves of
 * their FP32 spectra); 0: each member solves its own systems inside its
 * branch, bit for bit as cf_time_step_rk3. */
int cf_ensemble_set_batched_tri(cf_ensemble *e, int on);
/* 1 (up to 32 members; default 0): the fused dynamic Smagorinsky pass of
 * every member that takes it (no wall model) and the fused right-hand sides
 * of all members run as one launch each per substep, every (member, tile) a
 * block of it -- per member the same arithmetic as its own launch; the
 * other kernels stay in the members' branches.  0: every kernel in the
 * members' branches. */
int cf_ensemble_set_batched_stencils(cf_ensemble *e, int on);
/* Empirical choice of how the ensemble runs its stencil passes and its
 * tridiagonal solves: one whole ensemble step per candidate captures its
 * graph, then `steps` steps are timed (CUDA events).  Candidates 0-3: each
 * member solves its own tridiagonal systems (as cf_time_step_rk3); 4-7: one
 * FP64 launch for all members' systems.  Within each group: (+0) every
 * kernel in the members' branches with each member's own z-chunk plan, and
 * the batched DSM / right-hand-side launches with (+1) the members' plans,
 * (+2) one z chunk per member, (+3) two.  The fastest is kept.  The ensemble
 * advances CF_ENS_TUNE_CANDIDATES (steps + 1) steps.  report
 * (CF_ENS_TUNE_CANDIDATES doubles, may be NULL): ms per step of each
 * candidate; choice (may be NULL): the one kept. */
enum { CF_ENS_TUNE_CANDIDATES = 8 };
int cf_ensemble_autotune(cf_ensemble *e, int steps, double *report, int *choice);

/* ---- divergence check without device allocation ---------------------- */
/* No counterpart in the reference: the arithmetic is check_divergence
 * (projection.f90:234-256), as in cf_check_divergence, but on caller-owned
 * device arrays, with no context and no device allocation.  It serves callers
 * that must not allocate device memory while they run -- all device memory
 * handed to their own pool at start-up, a fixed memory cap, or no room for the
 * device synchronisation a cudaMalloc/cudaFree may cause -- and therefore
 * cannot call cf_create.
 *   U, V, W  device arrays, reference layout and extents (top of this file)
 *   x, y, z  face coordinates on the device (nx, ny, nz doubles)
 *   out      2 device doubles: max(0, max div) and max |div| over the interior
 *            cells i = 2..nx, j = 2..ny, k = 2..nz; both NaN when the
 *            divergence of any of those cells is NaN
 *   stream   a cudaStream_t (NULL: the legacy default stream); the work is
 *            enqueued on it and not waited for.
 * Scratch: one static device array per device holding CF_NOALLOC_MAX_PLANES
 * (max div, max |div|) pairs, one per interior z plane; nz - 1 above that is
 * rejected with CF_ERR_INVALID.  Nothing has to start at zero: every call
 * writes each scratch slot before it reads it.  Pointers that are not device
 * or managed memory of the current device are rejected.  The first call on
 * each device does a one-time setup (it looks up the scratch address with that
 * device current, which may load the library's device code); a caller that
 * captures streams should make that first call before any capture begins.
 * Calls that overlap on one device (several streams or host threads) share the
 * scratch and race: serialise them.  Errors: cf_last_error(NULL). */
enum { CF_NOALLOC_MAX_PLANES = 4096 };
int cf_check_divergence_noalloc(int nx, int ny, int nz, const double *U, const double *V, const double *W,
                                const double *x, const double *y, const double *z, double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
