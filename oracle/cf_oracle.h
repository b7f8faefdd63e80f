/*
 * cf_oracle.h -- CPU FP64 oracle for the RK3 substep of the staggered
 * finite-difference channel solver (Adrian-Lozano/channel-flow).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against, and the timed CPU baseline ("port" of the reference
 * CPU path).  The product (libchannel_gpu.so) never links, loads or calls it.
 *
 * Parity status: UNPINNED.  The reference is Fortran-90 + MPI + FFTW-MPI +
 * LAPACK and has no tests, fixtures or golden vectors; no Fortran compiler
 * exists in the build container, so the reference cannot be run to pin this
 * restatement.  Its third-party arithmetic (FFTW's DFT and LAPACK zgtsv) is
 * pinned separately against numpy.fft and scipy.linalg.lapack.zgtsv.
 *
 * Semantics: one process holding the whole domain, i.e. the reference's
 * multi-rank (nprocs >= 2) behaviour where the z-periodic exchange is a plain
 * wrap (boundary_conditions.f90:111-244).  All arrays use the reference's
 * Fortran extents and column-major order, ghosts and periodic duplicates
 * included (initialization.f90:121-152).
 */
#ifndef CF_ORACLE_H
#define CF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cfo cfo;

/* Scalar inputs of read_input_parameters (input_output.f90:21-133). */
typedef struct {
    double nu;            /* viscosity                                   */
    double CFL;           /* CFL (<0 -> fixed dt = -CFL)                 */
    double dPdx, dPdz;    /* pressure gradients                          */
    double Rossby_plus;   /* Omega_z = Rossby_plus*sqrt(dPdx)/2          */
    double freq_mult;     /* Ucenterline_x target when x_mass_cte == 2   */
    int Retau_int;        /* mass-flow rescale flag                      */
    int x_mass_cte, y_mass_cte;
    int LES_model;        /* 0 none, 2 dynamic Smagorinsky               */
    int iwall_model;      /* 0 no-slip, 3 equilibrium wall model         */
    int Dirichlet_nu_t;   /* 1 Dirichlet, 0 Neumann ghost for nu_t       */
    int jref_eqwm;        /* matching index for eqwm                     */
    int eqwm_ncv;         /* ODE cells; 100 in wallmodel.f90:621         */
    double eqwm_stretch;  /* ODE stretching; 1.10 in wallmodel.f90:621   */
} cfo_params;

/* Create from face grids x[nx], y[ny], z[nz] (global, 1 rank). */
cfo *cfo_create(int nx, int ny, int nz, const double *x, const double *y,
                const double *z, const cfo_params *p);
void cfo_destroy(cfo *o);

/* Copy fields in/out, Fortran layout with reference extents:
 * U (nx,nyg,nzg), V (nxg,ny,nzg), W (nxg,nyg,nz), P and nu_t (nxg,nyg,nzg). */
void cfo_set_fields(cfo *o, const double *U, const double *V, const double *W);
void cfo_get_fields(cfo *o, double *U, double *V, double *W, double *P, double *nu_t);

/* Raw access to a named internal array (for tests); returns NULL if unknown.
 * dims[0..3] receive the extents (1 for unused dims). */
double *cfo_array(cfo *o, const char *name, int *dims);
double cfo_scalar(cfo *o, const char *name);
void cfo_set_scalar(cfo *o, const char *name, double v);

/* initialization.f90:432-463 (initial mass flow, Retau rescale) */
void cfo_init_mass_flow(cfo *o);

/* Mirrors of the reference subroutines. */
void cfo_compute_dt(cfo *o);                       /* time_integration.f90:179 */
void cfo_time_step_rk3(cfo *o);                    /* time_integration.f90:89  */
void cfo_compute_eddy_viscosity(cfo *o);           /* subgrid.f90:23           */
void cfo_compute_wall_model(cfo *o);               /* wallmodel.f90:24         */
void cfo_compute_rhs_u(cfo *o, int slot);          /* equations.f90:24  -> Fu{slot} */
void cfo_compute_rhs_v(cfo *o, int slot);          /* equations.f90:186 -> Fv{slot} */
void cfo_compute_rhs_w(cfo *o, int slot);          /* equations.f90:351 -> Fw{slot} */
void cfo_rk_update(cfo *o, int substep);           /* time_integration.f90:108-146 */
void cfo_apply_boundary_conditions(cfo *o);        /* boundary_conditions.f90:20 */
void cfo_compute_projection_step(cfo *o);          /* projection.f90:20        */
void cfo_compute_pressure(cfo *o);                 /* pressure.f90:21          */
void cfo_compute_pseudo_pressure_rhs(cfo *o);      /* projection.f90:40        */
void cfo_solve_poisson_equation(cfo *o);           /* projection.f90:74        */
void cfo_project_velocity(cfo *o);                 /* projection.f90:203       */
double cfo_check_divergence(cfo *o, double *maxabs); /* projection.f90:234    */
double cfo_compute_dPx_for_constant_mass_flow(cfo *o); /* mass_flow.f90:103   */
double cfo_compute_mean_mass_flow_U(cfo *o);       /* mass_flow.f90:25         */
double cfo_compute_mean_mass_flow_V(cfo *o);       /* mass_flow.f90:61         */
void cfo_compute_statistics(cfo *o, double *out);  /* statistics.f90:43-155    */
void cfo_output_monitor(cfo *o, double *out);       /* monitor.f90:28-52        */
/* solve_u_eqwm (eqwm.f90:90-223) for one point: u_les, nu, matching height,
 * ODE cells and stretching, warm-start stress; returns tau_w, *iter the
 * Picard passes (101 = not converged). */
double cfo_solve_u_eqwm(double umag_les, double nu, double h_wm, int ncv, double stretch, double tau_in, int *iter);

/* Third-party arithmetic restated for pinning tests. */
void cfo_fft(double *re_im, int n, int sign);      /* complex DFT, FFTW sign   */
int cfo_zgtsv(int n, double *dl, double *d, double *du, double *b); /* complex,
        interleaved re/im, LAPACK zgtsv algorithm, one right-hand side */

/* Threads used by loops (OpenMP build); returns the active count. */
int cfo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
