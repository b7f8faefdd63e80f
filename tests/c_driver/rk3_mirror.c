/*
 * rk3_mirror.c -- a C caller of libchannel_gpu that advances a channel by
 * the reference's compute_time_step_RK3 (time_integration.f90:89-173) issued
 * call by call through the mirror entry points, in the reference's order,
 * and the same channel by the graph-captured cf_time_step_rk3, then prints
 * the normwise relative differences of U, V, W, P and nu_t as one JSON line.
 *
 * The initial fields come from a snapshot in the reference's format
 * (input_output.f90:231-384), read with cf_read_snapshot.
 *
 *   rk3_mirror SNAPSHOT NX NY NZ NU DPDX LES_MODEL IWALL_MODEL JREF NCV X_MASS_CTE Y_MASS_CTE DT NSTEPS PRECISION
 *
 * Exit status 0 when every call succeeded (the comparison is the caller's).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "channel_gpu.h"

#define CHECK(ctx, call)                                                                  \
    do {                                                                                  \
        int rc_ = (call);                                                                 \
        if (rc_ != CF_OK) {                                                               \
            fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, cf_last_error(ctx));      \
            exit(1);                                                                      \
        }                                                                                 \
    } while (0)

/* compute_dt, then compute_time_step_RK3 through the mirrors:
 *   to = t; Uo = U                                   (cf_save_old_state)
 *   per substep s: rk_step = s; eddy viscosity (s = 1: eddy viscosity, wall
 *   model, eddy viscosity); rhs_u, rhs_v, rhs_w into F{s}; U = Uo + dt*sum
 *   (cf_rk_update); t = to + rk_t(s)*dt; BCs; projection; BCs
 *   mass flow: x_mass_cte 1 or 2, then y_mass_cte 1, each followed by BCs */
static void mirror_step(cf_ctx *c, const cf_params *p) {
    static const double rk_t[3] = {8.0 / 15.0, 2.0 / 3.0, 1.0};
    double t, dt, dPdx, dPdy, d;
    int rk;
    CHECK(c, cf_compute_dt(c, &dt));
    CHECK(c, cf_get_scalars(c, &t, &dt, &rk, &dPdx, &dPdy));
    const double to = t;
    CHECK(c, cf_save_old_state(c));
    for (int s = 1; s <= 3; s++) {
        CHECK(c, cf_get_scalars(c, &t, &dt, &rk, &dPdx, &dPdy));
        CHECK(c, cf_set_scalars(c, t, dt, s, dPdx, dPdy));
        CHECK(c, cf_compute_eddy_viscosity(c));
        if (s == 1) {
            CHECK(c, cf_compute_wall_model(c));
            CHECK(c, cf_compute_eddy_viscosity(c));
        }
        CHECK(c, cf_compute_rhs_u(c, s));
        CHECK(c, cf_compute_rhs_v(c, s));
        CHECK(c, cf_compute_rhs_w(c, s));
        CHECK(c, cf_rk_update(c, s));
        CHECK(c, cf_set_scalars(c, to + rk_t[s - 1] * dt, dt, s, dPdx, dPdy));
        CHECK(c, cf_apply_boundary_conditions(c));
        CHECK(c, cf_compute_projection_step(c));
        CHECK(c, cf_apply_boundary_conditions(c));
    }
    if (p->x_mass_cte == 1 || p->x_mass_cte == 2) {
        if (p->x_mass_cte == 1) CHECK(c, cf_compute_dPx_for_constant_mass_flow(c, &d));
        else CHECK(c, cf_compute_dPx_for_constant_Ucenterline(c, &d));
        CHECK(c, cf_apply_mass_flow_correction(c, 0, d));
        CHECK(c, cf_apply_boundary_conditions(c));
    }
    if (p->y_mass_cte == 1) {
        CHECK(c, cf_compute_dPy_for_constant_mass_flow(c, &d));
        CHECK(c, cf_apply_mass_flow_correction(c, 1, d));
        CHECK(c, cf_apply_boundary_conditions(c));
    }
}

static double rel_err(const double *a, const double *b, size_t n) {
    double num = 0.0, den = 0.0;
    for (size_t q = 0; q < n; q++) {
        const double e = fabs(a[q] - b[q]), m = fabs(b[q]);
        if (e > num || isnan(e)) num = e;
        if (m > den) den = m;
    }
    return den > 0.0 ? num / den : num;
}

int main(int argc, char **argv) {
    if (argc != 16) {
        fprintf(stderr, "usage: %s SNAPSHOT NX NY NZ NU DPDX LES IWALL JREF NCV XMASS YMASS DT NSTEPS PRECISION\n",
                argv[0]);
        return 2;
    }
    const int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]);
    cf_params p;
    cf_default_params(&p);
    p.nu = atof(argv[5]);
    p.dPdx = atof(argv[6]);
    p.LES_model = atoi(argv[7]);
    p.iwall_model = atoi(argv[8]);
    p.jref_eqwm = atoi(argv[9]);
    p.eqwm_ncv = atoi(argv[10]);
    p.x_mass_cte = atoi(argv[11]);
    p.y_mass_cte = atoi(argv[12]);
    const double dt = atof(argv[13]);
    p.CFL = -dt; /* the reference's CFL < 0 rule: dt = -CFL */
    const int nsteps = atoi(argv[14]);
    p.precision = atoi(argv[15]);

    const size_t nxg = nx + 1, nyg = ny + 1, nzg = nz + 1;
    const size_t nU = nx * nyg * nzg, nV = nxg * ny * nzg, nW = nxg * nyg * nz, nP = nxg * nyg * nzg;
    double *x = malloc(nx * sizeof(double)), *y = malloc(ny * sizeof(double)), *z = malloc(nz * sizeof(double));
    double *U = malloc(nU * sizeof(double)), *V = malloc(nV * sizeof(double)), *W = malloc(nW * sizeof(double));
    if (cf_read_snapshot(argv[1], nx, ny, nz, x, y, z, U, V, W) != CF_OK) {
        fprintf(stderr, "cf_read_snapshot: %s\n", cf_last_error(NULL));
        return 1;
    }
    cf_ctx *ctx[2];
    double q0 = 0.0;
    for (int r = 0; r < 2; r++) {
        if (cf_create(nx, ny, nz, x, y, z, &p, 0, &ctx[r]) != CF_OK) {
            fprintf(stderr, "cf_create: %s\n", cf_last_error(NULL));
            return 1;
        }
        CHECK(ctx[r], cf_upload_fields(ctx[r], U, V, W));
        CHECK(ctx[r], cf_init_mass_flow(ctx[r], r == 0 ? &q0 : NULL));
        CHECK(ctx[r], cf_apply_boundary_conditions(ctx[r]));
        CHECK(ctx[r], cf_set_scalars(ctx[r], 0.0, dt, 1, p.dPdx, 0.0));
        CHECK(ctx[r], cf_set_fixed_dt(ctx[r], dt));
    }
    for (int s = 0; s < nsteps; s++) mirror_step(ctx[0], &p);
    CHECK(ctx[1], cf_time_step_rk3(ctx[1], nsteps, 1));

    double *out[2][5];
    const size_t sz[5] = {nU, nV, nW, nP, nP};
    for (int r = 0; r < 2; r++) {
        for (int f = 0; f < 5; f++) out[r][f] = malloc(sz[f] * sizeof(double));
        CHECK(ctx[r], cf_download_fields(ctx[r], out[r][0], out[r][1], out[r][2], out[r][3], out[r][4]));
    }
    double sc[2][4];
    for (int r = 0; r < 2; r++) {
        int rk;
        CHECK(ctx[r], cf_get_scalars(ctx[r], &sc[r][0], &sc[r][1], &rk, &sc[r][2], &sc[r][3]));
    }
    static const char *names[5] = {"U", "V", "W", "P", "nu_t"};
    printf("{");
    for (int f = 0; f < 5; f++) printf("\"%s\": %.6e, ", names[f], rel_err(out[0][f], out[1][f], sz[f]));
    printf("\"t\": [%.17g, %.17g], \"dPdx\": [%.17g, %.17g], \"Qflow_x_0\": %.17g}\n", sc[0][0], sc[1][0], sc[0][2],
           sc[1][2], q0);
    for (int r = 0; r < 2; r++) {
        for (int f = 0; f < 5; f++) free(out[r][f]);
        CHECK(ctx[r], cf_destroy(ctx[r]));
    }
    free(x); free(y); free(z); free(U); free(V); free(W);
    return 0;
}
