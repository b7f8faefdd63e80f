/*
 * cf_oracle.c -- CPU FP64 restatement of the reference RK3 substep.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).
 * Parity status: UNPINNED -- see cf_oracle.h.
 *
 * Every routine follows the Fortran of Adrian-Lozano/channel-flow loop for
 * loop; the citations name the reference file:line each block restates.
 * Array extents and lower bounds are the reference's, including the ghost
 * layers and the periodic duplicate planes, so values computed at duplicate
 * positions (which the reference does not always keep periodic, e.g. the
 * eqwm Neumann ghosts) are reproduced exactly.
 *
 * The whole domain is one slab: the z-periodic exchange of
 * boundary_conditions.f90:111-244 becomes a plain wrap (the reference's
 * nprocs >= 2 behaviour).  Reductions are computed per z-plane and summed in
 * plane order so that the result does not depend on the thread count.
 */
#include "cf_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Fortran-style arrays: column-major, arbitrary lower bounds.               */
/* ------------------------------------------------------------------------ */
typedef struct {
    double *p;
    int l[4], u[4];
    size_t n[4];
} fa;

static fa fa_new4(int l0, int u0, int l1, int u1, int l2, int u2, int l3, int u3) {
    fa a;
    a.l[0] = l0; a.u[0] = u0; a.l[1] = l1; a.u[1] = u1;
    a.l[2] = l2; a.u[2] = u2; a.l[3] = l3; a.u[3] = u3;
    size_t tot = 1;
    for (int d = 0; d < 4; d++) {
        a.n[d] = (size_t)(a.u[d] - a.l[d] + 1);
        tot *= a.n[d];
    }
    a.p = (double *)calloc(tot, sizeof(double));
    if (!a.p) { fprintf(stderr, "cf_oracle: out of memory\n"); abort(); }
    return a;
}
static fa fa_new3(int l0, int u0, int l1, int u1, int l2, int u2) {
    return fa_new4(l0, u0, l1, u1, l2, u2, 1, 1);
}
static void fa_free(fa *a) { free(a->p); a->p = NULL; }
static size_t fa_size(const fa *a) { return a->n[0] * a->n[1] * a->n[2] * a->n[3]; }

#ifdef CFO_CHECK
static size_t fa_idx(const fa *a, int i, int j, int k, int c, int line) {
    int v[4] = {i, j, k, c};
    for (int d = 0; d < 4; d++)
        if (v[d] < a->l[d] || v[d] > a->u[d]) {
            fprintf(stderr, "cf_oracle.c:%d index %d=%d outside [%d,%d]\n", line, d, v[d], a->l[d], a->u[d]);
            abort();
        }
    return (size_t)(i - a->l[0]) + a->n[0] * ((size_t)(j - a->l[1]) + a->n[1] * ((size_t)(k - a->l[2]) + a->n[2] * (size_t)(c - a->l[3])));
}
#define F3(a, i, j, k) ((a).p[fa_idx(&(a), (i), (j), (k), (a).l[3], __LINE__)])
#define F4(a, i, j, k, c) ((a).p[fa_idx(&(a), (i), (j), (k), (c), __LINE__)])
#else
#define F3(a, i, j, k) \
    ((a).p[(size_t)((i) - (a).l[0]) + (a).n[0] * ((size_t)((j) - (a).l[1]) + (a).n[1] * (size_t)((k) - (a).l[2]))])
#define F4(a, i, j, k, c)                                                                                    \
    ((a).p[(size_t)((i) - (a).l[0]) +                                                                         \
           (a).n[0] * ((size_t)((j) - (a).l[1]) + (a).n[1] * ((size_t)((k) - (a).l[2]) + (a).n[2] * (size_t)((c) - (a).l[3])))])
#endif

/* ------------------------------------------------------------------------ */
/* State: the module globals of global.f90:18-193 that the path touches.    */
/* ------------------------------------------------------------------------ */
struct cfo {
    cfo_params p;
    int nx, ny, nz, nxg, nyg, nzg, nxm, nym, nzm, nxp, nzp, mx, mz;
    double *x, *y, *z, *xm, *ym, *zm, *xg, *yg, *zg; /* 1-based */
    double *weight_y_0, *weight_y_1;                  /* 1..ny    */
    double *kxx, *kzz;                                /* 0-based  */
    double dxmin, dymin, dzmin, dx, dz, Lx, Ly, Lz;
    fa Dyy; /* (2:nyg-1, 2:nyg-1) */
    double coef_bc_1, coef_bc_2;
    double rk_t[4], rk_coef[4][4];
    double nu, CFL, dPdx, dPdy, dPdz, dPdx_ref, Omega_z;
    double Qflow_x_0, Qflow_y_0, Ucenterline_x, tau_mean_eqwm, fil_size;
    double t, dt;
    int rk_step, istep;
    fa U, V, W, P, Uo, Vo, Wo, nu_t, avg_nu_t;
    fa Fu[4], Fv[4], Fw[4];
    fa rhs_p;
    fa term, term_1, term_2;
    fa Lij, Mij, Sij, S, ten_buf, Uf, Vf, Wf, Sc;
    fa alpha_x, alpha_y, alpha_z, alpha_z_temp, tau_eqwm_initial;
    fa temp_1, temp_2, temp_3, temp_4;
    int n_nan_eqwm, n_iter_eqwm;
    int amd_nan_canonical; /* canonical cells of the last sgs_AMD whose quotient was NaN */
    double complex *plane; /* nxp*nzp spectrum plane */
    double complex *rhs_p_hat; /* (0:mx, 2:nyg-1, 0:mz) */
    double complex *twx_f, *twx_b, *twz_f, *twz_b; /* DFT twiddles */
};

static double *vec1(int n) { /* 1-based vector of length n */
    double *v = (double *)calloc((size_t)n + 2, sizeof(double));
    if (!v) abort();
    return v;
}

int cfo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Complex DFT (FFTW sign convention, unnormalised): a plain mixed-radix     */
/* Cooley-Tukey recursion; restates the transform FFTW computes at           */
/* projection.f90:85,118.                                                    */
/* ------------------------------------------------------------------------ */
/* tw[e] = exp(sign*2*pi*i*e/N), e = 0..N-1; a level of size n (n | N) uses
 * W_n^e = tw[(e mod n)*(N/n)]. */
static double complex *twiddles(int N, int sign) {
    double complex *tw = (double complex *)malloc(sizeof(double complex) * (size_t)N);
    for (int e = 0; e < N; e++) {
        double ang = sign * 2.0 * M_PI * (double)e / (double)N;
        tw[e] = cos(ang) + I * sin(ang);
    }
    return tw;
}

static void fft_rec(const double complex *in, size_t stride, double complex *out, int n, int N,
                    const double complex *tw, double complex *scratch) {
    if (n == 1) { out[0] = in[0]; return; }
    int p = 0;
    for (int f = 2; f * f <= n; f++) if (n % f == 0) { p = f; break; }
    if (p == 0) p = n; /* prime length: direct DFT */
    int m = n / p;
    size_t step = (size_t)(N / n);
    if (m == 1) {
        for (int k = 0; k < n; k++) {
            double complex s = 0;
            for (int r = 0; r < n; r++) s += in[(size_t)r * stride] * tw[(((size_t)r * k) % n) * step];
            out[k] = s;
        }
        return;
    }
    for (int r = 0; r < p; r++) fft_rec(in + (size_t)r * stride, stride * p, out + (size_t)r * m, m, N, tw, scratch + n);
    for (int k = 0; k < n; k++) scratch[k] = out[k];
    for (int k = 0; k < m; k++)
        for (int q = 0; q < p; q++) {
            int kk = k + q * m;
            double complex s = 0;
            for (int r = 0; r < p; r++) s += scratch[r * m + k] * tw[(((size_t)r * kk) % n) * step];
            out[kk] = s;
        }
}

static void fft_line(double complex *data, size_t stride, int n, const double complex *tw, double complex *work) {
    /* work holds n (input copy) + n (output) + 4n scratch */
    double complex *in = work, *out = work + n, *scr = work + 2 * n;
    for (int k = 0; k < n; k++) in[k] = data[(size_t)k * stride];
    fft_rec(in, 1, out, n, n, tw, scr);
    for (int k = 0; k < n; k++) data[(size_t)k * stride] = out[k];
}

void cfo_fft(double *re_im, int n, int sign) {
    double complex *work = (double complex *)malloc(sizeof(double complex) * (size_t)(8 * n + 8));
    double complex *tw = twiddles(n, sign < 0 ? -1 : 1);
    fft_line((double complex *)re_im, 1, n, tw, work);
    free(work);
    free(tw);
}

/* 2-D transform of a plane stored x-fastest (nxp, nzp). */
static void fft2d(double complex *pl, int nxp, int nzp, const double complex *twx, const double complex *twz) {
    int nmax = nxp > nzp ? nxp : nzp;
#pragma omp parallel
    {
        double complex *work = (double complex *)malloc(sizeof(double complex) * (size_t)(8 * nmax + 8));
#pragma omp for schedule(static)
        for (int k = 0; k < nzp; k++) fft_line(pl + (size_t)k * nxp, 1, nxp, twx, work);
#pragma omp for schedule(static)
        for (int i = 0; i < nxp; i++) fft_line(pl + i, (size_t)nxp, nzp, twz, work);
        free(work);
    }
}

/* ------------------------------------------------------------------------ */
/* LAPACK zgtsv (Gaussian elimination with partial pivoting), restated from  */
/* the published algorithm of LAPACK 3.2.1; called at projection.f90:110.    */
/* Complex entries; CABS1(z) = |Re z| + |Im z|.                              */
/* ------------------------------------------------------------------------ */
static inline double cabs1(double complex z) { return fabs(creal(z)) + fabs(cimag(z)); }

static int zgtsv_c(int n, double complex *dl, double complex *d, double complex *du, double complex *b) {
    if (n <= 0) return 0;
    for (int k = 0; k < n - 1; k++) {
        if (dl[k] == 0.0) {
            if (d[k] == 0.0) return k + 1;
        } else if (cabs1(d[k]) >= cabs1(dl[k])) {
            double complex mult = dl[k] / d[k];
            d[k + 1] = d[k + 1] - mult * du[k];
            b[k + 1] = b[k + 1] - mult * b[k];
            if (k < n - 2) dl[k] = 0.0;
        } else {
            double complex mult = d[k] / dl[k];
            d[k] = dl[k];
            double complex temp = d[k + 1];
            d[k + 1] = du[k] - mult * temp;
            if (k < n - 2) {
                dl[k] = du[k + 1];
                du[k + 1] = -mult * dl[k];
            }
            du[k] = temp;
            temp = b[k];
            b[k] = b[k + 1];
            b[k + 1] = temp - mult * b[k + 1];
        }
    }
    if (d[n - 1] == 0.0) return n;
    b[n - 1] = b[n - 1] / d[n - 1];
    if (n > 1) b[n - 2] = (b[n - 2] - du[n - 2] * b[n - 1]) / d[n - 2];
    for (int k = n - 3; k >= 0; k--) b[k] = (b[k] - du[k] * b[k + 1] - dl[k] * b[k + 2]) / d[k];
    return 0;
}

int cfo_zgtsv(int n, double *dl, double *d, double *du, double *b) {
    return zgtsv_c(n, (double complex *)dl, (double complex *)d, (double complex *)du, (double complex *)b);
}

/* ------------------------------------------------------------------------ */
/* Creation: grids and constants of initialization.f90:79-429.               */
/* ------------------------------------------------------------------------ */
static void build_ghost_grid(const double *f, int n, double *m, double *g) {
    /* initialization.f90:169-195 */
    for (int i = 1; i <= n - 1; i++) m[i] = 0.5 * (f[i] + f[i + 1]);
    for (int i = 1; i <= n - 1; i++) g[i + 1] = m[i];
    g[1] = m[1] - 2.0 * (m[1] - f[1]);
    g[n + 1] = m[n - 1] + 2.0 * (f[n] - m[n - 1]);
}

static void build_Dyy(cfo *o) {
    /* initialization.f90:343-373 */
    int nyg = o->nyg;
    double *y = o->y, *yg = o->yg;
    double a, b, c;
    for (size_t q = 0; q < fa_size(&o->Dyy); q++) o->Dyy.p[q] = 0.0;
    for (int j = 3; j <= nyg - 2; j++) {
        a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j]);
        b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]));
        c = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1]);
        F3(o->Dyy, j, j + 1, 1) = a;
        F3(o->Dyy, j, j - 1, 1) = c;
        F3(o->Dyy, j, j, 1) = b;
    }
    int j = 2;
    a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j]);
    b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]));
    c = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1]);
    F3(o->Dyy, 2, 2, 1) = b + c;
    F3(o->Dyy, 2, 3, 1) = a;
    o->coef_bc_1 = c;
    j = nyg - 1;
    a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j]);
    b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]));
    c = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1]);
    F3(o->Dyy, nyg - 1, nyg - 1, 1) = a + b;
    F3(o->Dyy, nyg - 1, nyg - 2, 1) = c;
    o->coef_bc_2 = a;
}

cfo *cfo_create(int nx, int ny, int nz, const double *x, const double *y, const double *z, const cfo_params *p) {
    if (nx % 2 || nz % 2 || nx < 6 || nz < 6 || ny < 4) return NULL; /* initialization.f90:54-62 */
    cfo *o = (cfo *)calloc(1, sizeof(cfo));
    o->p = *p;
    o->nx = nx; o->ny = ny; o->nz = nz;
    o->nxm = nx - 1; o->nym = ny - 1; o->nzm = nz - 1;          /* initialization.f90:84-90 */
    o->nxg = nx + 1; o->nyg = ny + 1; o->nzg = nz + 1;          /* initialization.f90:97-99 */
    o->nxp = o->nxm - 1; o->nzp = o->nzm - 1;                    /* initialization.f90:246-247 */
    o->mx = o->nxp - 1; o->mz = o->nzp - 1;
    int nxg = o->nxg, nyg = o->nyg, nzg = o->nzg;

    o->x = vec1(nx); o->y = vec1(ny); o->z = vec1(nz);
    o->xm = vec1(nx); o->ym = vec1(ny); o->zm = vec1(nz);
    o->xg = vec1(nxg); o->yg = vec1(nyg); o->zg = vec1(nzg);
    for (int i = 1; i <= nx; i++) o->x[i] = x[i - 1];
    for (int j = 1; j <= ny; j++) o->y[j] = y[j - 1];
    for (int k = 1; k <= nz; k++) o->z[k] = z[k - 1];
    build_ghost_grid(o->x, nx, o->xm, o->xg);
    build_ghost_grid(o->y, ny, o->ym, o->yg);
    build_ghost_grid(o->z, nz, o->zm, o->zg);

    /* initialization.f90:208-215 */
    o->dxmin = o->xg[2] - o->xg[1];
    for (int i = 1; i <= nxg - 1; i++) if (o->xg[i + 1] - o->xg[i] < o->dxmin) o->dxmin = o->xg[i + 1] - o->xg[i];
    o->dymin = o->yg[2] - o->yg[1];
    for (int j = 1; j <= nyg - 1; j++) if (o->yg[j + 1] - o->yg[j] < o->dymin) o->dymin = o->yg[j + 1] - o->yg[j];
    o->dzmin = o->zg[2] - o->zg[1];
    for (int k = 1; k <= nzg - 1; k++) if (o->zg[k + 1] - o->zg[k] < o->dzmin) o->dzmin = o->zg[k + 1] - o->zg[k];
    o->Lx = o->x[nx] - o->x[1];
    o->Ly = o->y[ny] - o->y[1];
    o->Lz = o->z[nz] - o->z[1];

    /* modified wavenumbers, initialization.f90:238-296 */
    o->dx = o->dxmin;
    o->dz = o->dzmin;
    double pi = 4.0 * atan(1.0);
    o->kxx = (double *)calloc((size_t)o->nxp, sizeof(double));
    o->kzz = (double *)calloc((size_t)o->nzp, sizeof(double));
    int hx = (int)ceil((double)(float)o->nxp / 2.0), hz = (int)ceil((double)(float)o->nzp / 2.0);
    for (int i = 0; i <= hx && i <= o->mx; i++)
        o->kxx[i] = 2.0 * (cos(2.0 * pi * (double)i / (double)o->nxp) - 1.0) / pow(o->dx, 2.0);
    for (int i = hx + 1; i <= o->mx; i++)
        o->kxx[i] = 2.0 * (cos(2.0 * pi * (double)(-o->nxp + i) / (double)o->nxp) - 1.0) / pow(o->dx, 2.0);
    for (int k = 0; k <= hz && k <= o->mz; k++)
        o->kzz[k] = 2.0 * (cos(2.0 * pi * (double)k / (double)o->nzp) - 1.0) / pow(o->dz, 2.0);
    for (int k = hz + 1; k <= o->mz; k++)
        o->kzz[k] = 2.0 * (cos(2.0 * pi * (double)(-o->nzp + k) / (double)o->nzp) - 1.0) / pow(o->dz, 2.0);

    o->Dyy = fa_new3(2, nyg - 1, 2, nyg - 1, 1, 1);
    build_Dyy(o);

    /* initialization.f90:386-388 */
    o->weight_y_0 = vec1(ny);
    o->weight_y_1 = vec1(ny);
    for (int j = 1; j <= ny; j++) {
        o->weight_y_0[j] = (o->yg[j + 1] - o->y[j]) / (o->yg[j + 1] - o->yg[j]);
        o->weight_y_1[j] = 1.0 - o->weight_y_0[j];
    }

    /* initialization.f90:405-417 */
    o->rk_t[1] = 8.0 / 15.0; o->rk_t[2] = 2.0 / 3.0; o->rk_t[3] = 1.0;
    o->rk_coef[1][1] = 8.0 / 15.0;
    o->rk_coef[2][1] = 1.0 / 4.0; o->rk_coef[2][2] = 5.0 / 12.0;
    o->rk_coef[3][1] = 1.0 / 4.0; o->rk_coef[3][2] = 0.0; o->rk_coef[3][3] = 3.0 / 4.0;

    /* input_output.f90:83-85 */
    o->nu = p->nu; o->CFL = p->CFL; o->dPdx = p->dPdx; o->dPdz = p->dPdz;
    o->Omega_z = p->Rossby_plus * sqrt(p->dPdx) / 2.0;
    o->dPdx_ref = p->dPdx;
    o->dPdy = 0.0;
    o->tau_mean_eqwm = o->dPdx_ref; /* initialization.f90:524 */
    o->t = 0.0;

    /* arrays, initialization.f90:121-152,419-429,466-528 */
    o->U = fa_new3(1, nx, 1, nyg, 1, nzg);
    o->V = fa_new3(1, nxg, 1, ny, 1, nzg);
    o->W = fa_new3(1, nxg, 1, nyg, 1, nz);
    o->P = fa_new3(1, nxg, 1, nyg, 1, nzg);
    o->Uo = fa_new3(1, nx, 1, nyg, 1, nzg);
    o->Vo = fa_new3(1, nxg, 1, ny, 1, nzg);
    o->Wo = fa_new3(1, nxg, 1, nyg, 1, nz);
    o->nu_t = fa_new3(1, nxg, 1, nyg, 1, nzg);
    o->avg_nu_t = fa_new3(1, 1, 1, nyg, 1, 1);
    for (int s = 1; s <= 3; s++) {
        o->Fu[s] = fa_new3(2, nx - 1, 2, nyg - 1, 2, nzg - 1);
        o->Fv[s] = fa_new3(2, nxg - 1, 2, ny - 1, 2, nzg - 1);
        o->Fw[s] = fa_new3(2, nxg - 1, 2, nyg - 1, 2, nz - 1);
    }
    o->rhs_p = fa_new3(2, nxg - 1, 2, nyg - 1, 2, nzg);
    o->term = fa_new3(1, nxg, 1, nyg, 1, nzg);
    o->term_1 = fa_new3(1, nxg, 1, nyg, 1, nzg);
    o->term_2 = fa_new3(1, nxg, 1, nyg, 1, nzg);
    if (p->LES_model > 0) {
        o->Lij = fa_new4(2, nxg, 2, nyg - 1, 2, nzg, 1, 6);
        o->Mij = fa_new4(2, nxg - 1, 2, nyg - 1, 2, nzg - 1, 1, 6);
        o->Sij = fa_new4(2, nxg, 2, nyg, 2, nzg, 1, 6);
        o->S = fa_new3(2, nxg - 1, 2, nyg - 1, 2, nzg - 1);
        o->Sc = fa_new4(2, nxg - 1, 2, nyg - 1, 2, nzg - 1, 1, 3);
        o->ten_buf = fa_new4(1, nxg, 1, nyg, 1, nzg, 1, 6);
        o->Uf = fa_new3(1, nx, 1, nyg, 1, nzg);
        o->Vf = fa_new3(1, nxg, 1, ny, 1, nzg);
        o->Wf = fa_new3(1, nxg, 1, nyg, 1, nz);
    }
    o->alpha_x = fa_new3(1, nx, 1, 2, 1, nzg);
    o->alpha_y = fa_new3(1, nxg, 1, 2, 1, nzg);
    o->alpha_z = fa_new3(1, nxg, 1, 2, 1, nz);
    o->alpha_z_temp = fa_new3(1, nx, 1, 2, 1, nzg);
    o->tau_eqwm_initial = fa_new3(1, nx, 1, 2, 1, nzg);
    for (size_t q = 0; q < fa_size(&o->tau_eqwm_initial); q++) o->tau_eqwm_initial.p[q] = o->tau_mean_eqwm;
    o->temp_1 = fa_new3(1, nxg, 1, 1, 1, nzg);
    o->temp_2 = fa_new3(1, nx, 1, 1, 1, nzg);
    o->temp_3 = fa_new3(1, nxg, 1, 1, 1, nz);
    o->temp_4 = fa_new3(1, nx, 1, 1, 1, nzg);
    o->plane = (double complex *)calloc((size_t)o->nxp * o->nzp, sizeof(double complex));
    o->rhs_p_hat = (double complex *)calloc((size_t)o->nxp * o->nym * o->nzp, sizeof(double complex));
    o->twx_f = twiddles(o->nxp, -1); o->twx_b = twiddles(o->nxp, 1);
    o->twz_f = twiddles(o->nzp, -1); o->twz_b = twiddles(o->nzp, 1);
    return o;
}

void cfo_destroy(cfo *o) {
    if (!o) return;
    fa *all[] = {&o->Dyy, &o->U, &o->V, &o->W, &o->P, &o->Uo, &o->Vo, &o->Wo, &o->nu_t, &o->avg_nu_t,
                 &o->rhs_p, &o->term, &o->term_1, &o->term_2, &o->Lij, &o->Mij, &o->Sij, &o->S, &o->ten_buf,
                 &o->Uf, &o->Vf, &o->Wf, &o->Sc, &o->alpha_x, &o->alpha_y, &o->alpha_z, &o->alpha_z_temp,
                 &o->tau_eqwm_initial, &o->temp_1, &o->temp_2, &o->temp_3, &o->temp_4};
    for (size_t q = 0; q < sizeof(all) / sizeof(all[0]); q++) fa_free(all[q]);
    for (int s = 1; s <= 3; s++) { fa_free(&o->Fu[s]); fa_free(&o->Fv[s]); fa_free(&o->Fw[s]); }
    free(o->x); free(o->y); free(o->z); free(o->xm); free(o->ym); free(o->zm);
    free(o->xg); free(o->yg); free(o->zg); free(o->weight_y_0); free(o->weight_y_1);
    free(o->kxx); free(o->kzz); free(o->plane); free(o->rhs_p_hat);
    free(o->twx_f); free(o->twx_b); free(o->twz_f); free(o->twz_b);
    free(o);
}

void cfo_set_fields(cfo *o, const double *U, const double *V, const double *W) {
    memcpy(o->U.p, U, fa_size(&o->U) * sizeof(double));
    memcpy(o->V.p, V, fa_size(&o->V) * sizeof(double));
    memcpy(o->W.p, W, fa_size(&o->W) * sizeof(double));
    /* input_output.f90:380-382 */
    memcpy(o->Uo.p, U, fa_size(&o->U) * sizeof(double));
    memcpy(o->Vo.p, V, fa_size(&o->V) * sizeof(double));
    memcpy(o->Wo.p, W, fa_size(&o->W) * sizeof(double));
}

void cfo_get_fields(cfo *o, double *U, double *V, double *W, double *P, double *nu_t) {
    if (U) memcpy(U, o->U.p, fa_size(&o->U) * sizeof(double));
    if (V) memcpy(V, o->V.p, fa_size(&o->V) * sizeof(double));
    if (W) memcpy(W, o->W.p, fa_size(&o->W) * sizeof(double));
    if (P) memcpy(P, o->P.p, fa_size(&o->P) * sizeof(double));
    if (nu_t) memcpy(nu_t, o->nu_t.p, fa_size(&o->nu_t) * sizeof(double));
}

double *cfo_array(cfo *o, const char *name, int *dims) {
    struct { const char *n; fa *a; } tab[] = {
        {"U", &o->U}, {"V", &o->V}, {"W", &o->W}, {"P", &o->P}, {"Uo", &o->Uo}, {"Vo", &o->Vo}, {"Wo", &o->Wo},
        {"nu_t", &o->nu_t}, {"avg_nu_t", &o->avg_nu_t}, {"rhs_p", &o->rhs_p},
        {"Fu1", &o->Fu[1]}, {"Fu2", &o->Fu[2]}, {"Fu3", &o->Fu[3]},
        {"Fv1", &o->Fv[1]}, {"Fv2", &o->Fv[2]}, {"Fv3", &o->Fv[3]},
        {"Fw1", &o->Fw[1]}, {"Fw2", &o->Fw[2]}, {"Fw3", &o->Fw[3]},
        {"Lij", &o->Lij}, {"Mij", &o->Mij}, {"Sij", &o->Sij}, {"S", &o->S},
        {"Uf", &o->Uf}, {"Vf", &o->Vf}, {"Wf", &o->Wf}, {"Dyy", &o->Dyy},
        {"alpha_x", &o->alpha_x}, {"alpha_y", &o->alpha_y}, {"alpha_z", &o->alpha_z},
        {"tau_eqwm_initial", &o->tau_eqwm_initial}, {"temp_2", &o->temp_2}, {"temp_4", &o->temp_4},
    };
    for (size_t q = 0; q < sizeof(tab) / sizeof(tab[0]); q++)
        if (strcmp(tab[q].n, name) == 0) {
            if (!tab[q].a->p) return NULL;
            for (int d = 0; d < 4; d++) dims[d] = (int)tab[q].a->n[d];
            return tab[q].a->p;
        }
    struct { const char *n; double *v; int len; } vt[] = {
        {"x", o->x + 1, o->nx}, {"y", o->y + 1, o->ny}, {"z", o->z + 1, o->nz},
        {"xg", o->xg + 1, o->nxg}, {"yg", o->yg + 1, o->nyg}, {"zg", o->zg + 1, o->nzg},
        {"kxx", o->kxx, o->nxp}, {"kzz", o->kzz, o->nzp},
        {"weight_y_0", o->weight_y_0 + 1, o->ny}, {"weight_y_1", o->weight_y_1 + 1, o->ny},
    };
    for (size_t q = 0; q < sizeof(vt) / sizeof(vt[0]); q++)
        if (strcmp(vt[q].n, name) == 0) {
            dims[0] = vt[q].len; dims[1] = dims[2] = dims[3] = 1;
            return vt[q].v;
        }
    return NULL;
}

double cfo_scalar(cfo *o, const char *name) {
    if (!strcmp(name, "dt")) return o->dt;
    if (!strcmp(name, "t")) return o->t;
    if (!strcmp(name, "dPdx")) return o->dPdx;
    if (!strcmp(name, "dPdy")) return o->dPdy;
    if (!strcmp(name, "dPdz")) return o->dPdz;
    if (!strcmp(name, "Qflow_x_0")) return o->Qflow_x_0;
    if (!strcmp(name, "Omega_z")) return o->Omega_z;
    if (!strcmp(name, "rk_step")) return o->rk_step;
    if (!strcmp(name, "n_nan_eqwm")) return o->n_nan_eqwm;
    if (!strcmp(name, "amd_nan_canonical")) return o->amd_nan_canonical;
    if (!strcmp(name, "n_iter_eqwm")) return o->n_iter_eqwm;
    if (!strcmp(name, "tau_mean_eqwm")) return o->tau_mean_eqwm;
    if (!strcmp(name, "dxmin")) return o->dxmin;
    if (!strcmp(name, "dymin")) return o->dymin;
    if (!strcmp(name, "dzmin")) return o->dzmin;
    if (!strcmp(name, "istep")) return o->istep;
    return NAN;
}

void cfo_set_scalar(cfo *o, const char *name, double v) {
    if (!strcmp(name, "dt")) o->dt = v;
    else if (!strcmp(name, "t")) o->t = v;
    else if (!strcmp(name, "dPdx")) o->dPdx = v;
    else if (!strcmp(name, "dPdz")) o->dPdz = v;
    else if (!strcmp(name, "Qflow_x_0")) o->Qflow_x_0 = v;
    else if (!strcmp(name, "rk_step")) o->rk_step = (int)v;
    else if (!strcmp(name, "istep")) o->istep = (int)v;
    else if (!strcmp(name, "tau_mean_eqwm")) o->tau_mean_eqwm = v;
}

/* ------------------------------------------------------------------------ */
/* Mass flow, mass_flow.f90                                                  */
/* ------------------------------------------------------------------------ */
double cfo_compute_mean_mass_flow_U(cfo *o) {
    /* mass_flow.f90:25-52; per-plane partials summed in plane order */
    int nx = o->nx, nyg = o->nyg, nzg = o->nzg;
    double *qk = (double *)calloc((size_t)nzg + 1, sizeof(double)), *nk = (double *)calloc((size_t)nzg + 1, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++) {
        double q = 0.0, n = 0.0;
        for (int j = 3; j <= nyg - 1; j++)
            for (int i = 2; i <= nx - 1; i++) {
                q = q + (F3(o->U, i, j, k) + F3(o->U, i, j - 1, k)) * 0.5 * (o->yg[j] - o->yg[j - 1]);
                n = n + (1.0 + 1.0) * 0.5 * (o->yg[j] - o->yg[j - 1]);
            }
        qk[k] = q; nk[k] = n;
    }
    double Q = 0.0, N = 0.0;
    for (int k = 2; k <= nzg - 1; k++) { Q += qk[k]; N += nk[k]; }
    free(qk); free(nk);
    return Q / N;
}

double cfo_compute_mean_mass_flow_V(cfo *o) {
    /* mass_flow.f90:61-88 */
    int nxg = o->nxg, ny = o->ny, nzg = o->nzg;
    double Q = 0.0, N = 0.0;
    for (int k = 2; k <= nzg - 1; k++) {
        double q = 0.0, n = 0.0;
        for (int j = 2; j <= ny; j++)
            for (int i = 2; i <= nxg - 1; i++) {
                q = q + (F3(o->V, i, j, k) + F3(o->V, i, j - 1, k)) * 0.5 * (o->y[j] - o->y[j - 1]);
                n = n + (1.0 + 1.0) * 0.5 * (o->y[j] - o->y[j - 1]);
            }
        Q += q; N += n;
    }
    return Q / N;
}

double cfo_compute_dPx_for_constant_mass_flow(cfo *o) {
    /* mass_flow.f90:103-132 (same sums as compute_mean_mass_flow_U) */
    return o->Qflow_x_0 - cfo_compute_mean_mass_flow_U(o);
}

static double compute_dPx_for_constant_Ucenterline(cfo *o) {
    /* mass_flow.f90:192-211 */
    int j = (int)floor((double)(float)(o->ny / 2)) + 1;
    double s = 0.0;
    for (int k = 1; k <= o->nzg - 2; k++)
        for (int i = 1; i <= o->nx - 2; i++) s += F3(o->U, i, j, k);
    s = s / (double)((o->nx - 2) * (o->nzg - 2));
    return o->Ucenterline_x - s;
}

static double compute_dPy_for_constant_mass_flow(cfo *o) {
    /* mass_flow.f90:147-176 */
    return o->Qflow_y_0 - cfo_compute_mean_mass_flow_V(o);
}

void cfo_init_mass_flow(cfo *o) {
    /* initialization.f90:432-463 */
    o->Qflow_x_0 = cfo_compute_mean_mass_flow_U(o);
    if (abs(o->p.Retau_int) > 0) {
        if (o->p.x_mass_cte == 1) {
            double Qflow_ref;
            switch (o->p.Retau_int) {
            case 4200: Qflow_ref = 0.873791265477842; break;
            case 2000: Qflow_ref = 0.898245304195718; break;
            case 950: Qflow_ref = 0.899952805947840; break;
            case 550: Qflow_ref = 0.899885379198784; break;
            case 395: Qflow_ref = 0.871974131836648; break;
            default:
                if (o->p.Retau_int < 0) Qflow_ref = -o->p.Retau_int * o->Qflow_x_0;
                else { fprintf(stderr, "Error: Unknown mass flow correction\n"); abort(); }
            }
            double f = Qflow_ref / o->Qflow_x_0;
            for (size_t q = 0; q < fa_size(&o->U); q++) o->U.p[q] = f * o->U.p[q];
        } else if (o->p.x_mass_cte == 2) {
            o->Ucenterline_x = o->p.freq_mult;
        }
    }
    o->Qflow_x_0 = cfo_compute_mean_mass_flow_U(o);
    o->Qflow_y_0 = cfo_compute_mean_mass_flow_V(o);
    o->Qflow_y_0 = 0.0;
    o->dPdy = 0.0;
}

/* ------------------------------------------------------------------------ */
/* compute_dt, time_integration.f90:179-227                                  */
/* ------------------------------------------------------------------------ */
void cfo_compute_dt(cfo *o) {
    int nxg = o->nxg, nyg = o->nyg, nzg = o->nzg;
    double lU = 0.0, lV = 0.0, lW = 0.0;
    for (int i = 2; i <= nxg - 1; i++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int k = 2; k <= nzg - 1; k++) {
                double a = (o->xg[i + 1] - o->xg[i]) / fabs(F3(o->U, i, j, k));
                double b = (o->yg[j + 1] - o->yg[j]) / fabs(F3(o->V, i, j, k));
                double c = (o->zg[k + 1] - o->zg[k]) / fabs(F3(o->W, i, j, k));
                lU = a > lU ? a : lU;
                lV = b > lV ? b : lV;
                lW = c > lW ? c : lW;
            }
    double du = o->CFL * lU, dv = o->CFL * lV, dw = o->CFL * lW;
    double dt_conv = du;
    if (dv < dt_conv) dt_conv = dv;
    if (dw < dt_conv) dt_conv = dw;
    double vu = o->CFL * pow(o->dxmin, 2.0) / o->nu;
    double vv = o->CFL * pow(o->dymin, 2.0) / o->nu;
    double vw = o->CFL * pow(o->dzmin, 2.0) / o->nu;
    double dt_vis = vu;
    if (vv < dt_vis) dt_vis = vv;
    if (vw < dt_vis) dt_vis = vw;
    double dt = dt_conv < dt_vis ? dt_conv : dt_vis;
    double dt_max = 5e-3;
    dt = dt < dt_max ? dt : dt_max;
    if (o->CFL < 0) dt = -o->CFL;
    o->dt = dt;
}

/* ------------------------------------------------------------------------ */
/* Boundary conditions, boundary_conditions.f90                              */
/* ------------------------------------------------------------------------ */
/* x-periodicity, boundary_conditions.f90:87-106.  id 1: x faces, 2: centres */
static void periodic_x(fa *F, int id, int nx, int nxg, int c) {
    for (int k = F->l[2]; k <= F->u[2]; k++)
        for (int j = F->l[1]; j <= F->u[1]; j++) {
            if (id == 1) {
                F4(*F, 1, j, k, c) = F4(*F, nx - 1, j, k, c);
                F4(*F, nx, j, k, c) = F4(*F, 2, j, k, c);
            } else {
                F4(*F, 1, j, k, c) = F4(*F, nxg - 2, j, k, c);
                F4(*F, nxg - 1, j, k, c) = F4(*F, 2, j, k, c);
                F4(*F, nxg, j, k, c) = F4(*F, 3, j, k, c);
            }
        }
}
/* z-periodicity, boundary_conditions.f90:111-244 with a one-slab wrap.
 * id 3: z faces (W-like); 1,2,4: z centres. */
static void periodic_z(fa *F, int id, int nz, int nzg, int c) {
    for (int j = F->l[1]; j <= F->u[1]; j++)
        for (int i = F->l[0]; i <= F->u[0]; i++) {
            if (id == 3) {
                double we = F4(*F, i, j, nz - 1, c), wi = F4(*F, i, j, 2, c);
                F4(*F, i, j, 1, c) = we;
                F4(*F, i, j, nz, c) = wi;
            } else {
                double e = F4(*F, i, j, nzg - 2, c), i2 = F4(*F, i, j, 2, c), i3 = F4(*F, i, j, 3, c);
                F4(*F, i, j, 1, c) = e;
                F4(*F, i, j, nzg - 1, c) = i2;
                F4(*F, i, j, nzg, c) = i3;
            }
        }
}
/* boundary_conditions.f90:257-272 */
static void dirichlet_y(fa *F, int id, int ny, int nyg) {
    for (int k = F->l[2]; k <= F->u[2]; k++)
        for (int i = F->l[0]; i <= F->u[0]; i++) {
            if (id == 1) { F3(*F, i, 1, k) = 0.0; F3(*F, i, ny, k) = 0.0; }
            else { F3(*F, i, 1, k) = -F3(*F, i, 2, k); F3(*F, i, nyg, k) = -F3(*F, i, nyg - 1, k); }
        }
}
/* boundary_conditions.f90:284-299 */
static void neumann_y(fa *F, int id, int ny, int nyg) {
    for (int k = F->l[2]; k <= F->u[2]; k++)
        for (int i = F->l[0]; i <= F->u[0]; i++) {
            if (id == 1) { F3(*F, i, 1, k) = F3(*F, i, 2, k); F3(*F, i, ny, k) = F3(*F, i, ny - 1, k); }
            else { F3(*F, i, 1, k) = F3(*F, i, 2, k); F3(*F, i, nyg, k) = F3(*F, i, nyg - 1, k); }
        }
}
/* boundary_conditions.f90:311-327 (id 2, centres) */
static void nonzero_neumann_y(cfo *o, fa *F, fa *alpha) {
    int nyg = o->nyg;
    for (int k = F->l[2]; k <= F->u[2]; k++)
        for (int i = F->l[0]; i <= F->u[0]; i++) {
            F3(*F, i, 1, k) = F3(*F, i, 2, k) - (o->yg[2] - o->yg[1]) * F3(*alpha, i, 1, k);
            F3(*F, i, nyg, k) = F3(*F, i, nyg - 1, k) - (o->yg[nyg] - o->yg[nyg - 1]) * F3(*alpha, i, 2, k);
        }
}

void cfo_apply_boundary_conditions(cfo *o) {
    /* boundary_conditions.f90:20-75 */
    periodic_x(&o->U, 1, o->nx, o->nxg, 1);
    periodic_x(&o->V, 2, o->nx, o->nxg, 1);
    periodic_x(&o->W, 2, o->nx, o->nxg, 1);
    periodic_z(&o->U, 1, o->nz, o->nzg, 1);
    periodic_z(&o->V, 2, o->nz, o->nzg, 1);
    periodic_z(&o->W, 3, o->nz, o->nzg, 1);
    if (o->p.iwall_model == 0) dirichlet_y(&o->U, 2, o->ny, o->nyg);
    else nonzero_neumann_y(o, &o->U, &o->alpha_x);
    dirichlet_y(&o->V, 1, o->ny, o->nyg);
    if (o->p.iwall_model == 0) dirichlet_y(&o->W, 2, o->ny, o->nyg);
    else nonzero_neumann_y(o, &o->W, &o->alpha_z);
}

/* ------------------------------------------------------------------------ */
/* Right-hand sides, equations.f90                                           */
/* ------------------------------------------------------------------------ */
void cfo_compute_rhs_u(cfo *o, int slot) {
    /* equations.f90:24-179 */
    int nx = o->nx, nyg = o->nyg, nzg = o->nzg, ny = o->ny;
    fa *U = &o->U, *V = &o->V, *W = &o->W, *nt = &o->nu_t, *R = &o->Fu[slot];
    const double *x = o->x, *y = o->y, *z = o->z, *xg = o->xg, *yg = o->yg, *zg = o->zg;
    const double *w0 = o->weight_y_0, *w1 = o->weight_y_1;
    double nu = o->nu, dPdx = o->dPdx, Om = o->Omega_z;
    (void)ny;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++) {
        double dz_1 = zg[k] - zg[k - 1], dz_2 = zg[k + 1] - zg[k], dz_3 = z[k] - z[k - 1];
        for (int j = 2; j <= nyg - 1; j++) {
            double dy_3 = y[j] - y[j - 1];
            for (int i = 2; i <= nx - 1; i++) {
                /* 1) -du^2/dx (:43-57); interpolate_x (interpolation.f90:38) then square */
                double a = 0.5 * (F3(*U, i, j, k) + F3(*U, i + 1, j, k));
                double b = 0.5 * (F3(*U, i - 1, j, k) + F3(*U, i, j, k));
                a = a * a; b = b * b;
                double r = -(a - b) / (xg[i + 1] - xg[i]);
                /* 2) -duv/dy (:62-79); interpolate_y weighted (interpolation.f90:71) */
                double uy1 = w0[j] * F3(*U, i, j, k) + w1[j] * F3(*U, i, j + 1, k);
                double uy0 = w0[j - 1] * F3(*U, i, j - 1, k) + w1[j - 1] * F3(*U, i, j, k);
                double vx1 = 0.5 * (F3(*V, i, j, k) + F3(*V, i + 1, j, k));
                double vx0 = 0.5 * (F3(*V, i, j - 1, k) + F3(*V, i + 1, j - 1, k));
                r = r + (-(uy1 * vx1 - uy0 * vx0) / (y[j] - y[j - 1]));
                /* 3) -duw/dz (:84-101) */
                double uz1 = 0.5 * (F3(*U, i, j, k) + F3(*U, i, j, k + 1));
                double uz0 = 0.5 * (F3(*U, i, j, k - 1) + F3(*U, i, j, k));
                double wx1 = 0.5 * (F3(*W, i, j, k) + F3(*W, i + 1, j, k));
                double wx0 = 0.5 * (F3(*W, i, j, k - 1) + F3(*W, i + 1, j, k - 1));
                r = r + (-(uz1 * wx1 - uz0 * wx0) / (z[k] - z[k - 1]));
                /* 4) viscous (:108-163) */
                double dx_1 = x[i] - x[i - 1], dx_2 = x[i + 1] - x[i], dx_3 = xg[i + 1] - xg[i];
                double t2j = (F3(*U, i, j + 1, k) - F3(*U, i, j, k)) / (yg[j + 1] - yg[j]);
                double t2jm = (F3(*U, i, j, k) - F3(*U, i, j - 1, k)) / (yg[j] - yg[j - 1]);
                double nu_x1 = nu + F3(*nt, i, j, k);
                double nu_x2 = nu + F3(*nt, i + 1, j, k);
                double nu_y1 = nu + 0.5 * (w0[j - 1] * F3(*nt, i, j - 1, k) + w1[j - 1] * F3(*nt, i, j, k) +
                                           w0[j - 1] * F3(*nt, i + 1, j - 1, k) + w1[j - 1] * F3(*nt, i + 1, j, k));
                double nu_y2 = nu + 0.5 * (w0[j] * F3(*nt, i, j, k) + w1[j] * F3(*nt, i, j + 1, k) +
                                           w0[j] * F3(*nt, i + 1, j, k) + w1[j] * F3(*nt, i + 1, j + 1, k));
                double nu_z1 = nu + 0.25 * (F3(*nt, i, j, k) + F3(*nt, i, j, k - 1) + F3(*nt, i + 1, j, k) + F3(*nt, i + 1, j, k - 1));
                double nu_z2 = nu + 0.25 * (F3(*nt, i, j, k) + F3(*nt, i, j, k + 1) + F3(*nt, i + 1, j, k) + F3(*nt, i + 1, j, k + 1));
                double visc =
                    2.0 / dx_3 * (nu_x2 * (F3(*U, i + 1, j, k) - F3(*U, i, j, k)) / dx_2 - nu_x1 * (F3(*U, i, j, k) - F3(*U, i - 1, j, k)) / dx_1) +
                    1.0 / dy_3 * (nu_y2 * (t2j + (F3(*V, i + 1, j, k) - F3(*V, i, j, k)) / dx_2) -
                                  nu_y1 * (t2jm + (F3(*V, i + 1, j - 1, k) - F3(*V, i, j - 1, k)) / dx_1)) +
                    1.0 / dz_3 * (nu_z2 * ((F3(*U, i, j, k + 1) - F3(*U, i, j, k)) / dz_2 + (F3(*W, i + 1, j, k) - F3(*W, i, j, k)) / dx_2) -
                                  nu_z1 * ((F3(*U, i, j, k) - F3(*U, i, j, k - 1)) / dz_1 + (F3(*W, i + 1, j, k - 1) - F3(*W, i, j, k - 1)) / dx_1));
                r = r + visc;
                /* constant pressure gradient (:166) */
                r = r + dPdx;
                /* rotation (:169-177): term = interpolate_y(V,1) at centre j, then interpolate_x */
                if (fabs(Om) > 1e-6) {
                    double tv0 = 0.5 * (F3(*V, i, j - 1, k) + F3(*V, i, j, k));
                    double tv1 = 0.5 * (F3(*V, i + 1, j - 1, k) + F3(*V, i + 1, j, k));
                    r = r + 2.0 * Om * (0.5 * (tv0 + tv1));
                }
                F3(*R, i, j, k) = r;
            }
        }
    }
}

void cfo_compute_rhs_v(cfo *o, int slot) {
    /* equations.f90:186-344 */
    int nx = o->nx, nxg = o->nxg, ny = o->ny, nzg = o->nzg;
    fa *U = &o->U, *V = &o->V, *W = &o->W, *nt = &o->nu_t, *R = &o->Fv[slot];
    const double *x = o->x, *y = o->y, *z = o->z, *xg = o->xg, *yg = o->yg, *zg = o->zg;
    const double *w0 = o->weight_y_0, *w1 = o->weight_y_1;
    double nu = o->nu, Om = o->Omega_z;
    (void)nx;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++) {
        double dz_1 = zg[k] - zg[k - 1], dz_2 = zg[k + 1] - zg[k], dz_3 = z[k] - z[k - 1];
        for (int j = 2; j <= ny - 1; j++) {
            double dy_1 = y[j] - y[j - 1], dy_2 = y[j + 1] - y[j], dy_3 = yg[j + 1] - yg[j];
            for (int i = 2; i <= nxg - 1; i++) {
                /* 1) -dv^2/dy (:205-223) */
                double a = 0.5 * (F3(*V, i, j, k) + F3(*V, i, j + 1, k));
                double b = 0.5 * (F3(*V, i, j - 1, k) + F3(*V, i, j, k));
                a = a * a; b = b * b;
                double r = -(a - b) / (yg[j + 1] - yg[j]);
                /* 2) -duv/dx (:228-245) */
                double uy1 = w0[j] * F3(*U, i, j, k) + w1[j] * F3(*U, i, j + 1, k);
                double uy0 = w0[j] * F3(*U, i - 1, j, k) + w1[j] * F3(*U, i - 1, j + 1, k);
                double vx1 = 0.5 * (F3(*V, i, j, k) + F3(*V, i + 1, j, k));
                double vx0 = 0.5 * (F3(*V, i - 1, j, k) + F3(*V, i, j, k));
                r = r + (-(uy1 * vx1 - uy0 * vx0) / (x[i] - x[i - 1]));
                /* 3) -dvw/dz (:250-267) */
                double vz1 = 0.5 * (F3(*V, i, j, k) + F3(*V, i, j, k + 1));
                double vz0 = 0.5 * (F3(*V, i, j, k - 1) + F3(*V, i, j, k));
                double wy1 = w0[j] * F3(*W, i, j, k) + w1[j] * F3(*W, i, j + 1, k);
                double wy0 = w0[j] * F3(*W, i, j, k - 1) + w1[j] * F3(*W, i, j + 1, k - 1);
                r = r + (-(vz1 * wy1 - vz0 * wy0) / (z[k] - z[k - 1]));
                /* 4) viscous (:276-331) */
                double dx_1 = xg[i] - xg[i - 1], dx_2 = xg[i + 1] - xg[i], dx_3 = x[i] - x[i - 1];
                double nu_x1 = nu + 0.5 * (w0[j] * F3(*nt, i - 1, j, k) + w1[j] * F3(*nt, i - 1, j + 1, k) +
                                           w0[j] * F3(*nt, i, j, k) + w1[j] * F3(*nt, i, j + 1, k));
                double nu_x2 = nu + 0.5 * (w0[j] * F3(*nt, i, j, k) + w1[j] * F3(*nt, i, j + 1, k) +
                                           w0[j] * F3(*nt, i + 1, j, k) + w1[j] * F3(*nt, i + 1, j + 1, k));
                double nu_y1 = nu + F3(*nt, i, j, k);
                double nu_y2 = nu + F3(*nt, i, j + 1, k);
                double nu_z1 = nu + 0.5 * (w0[j] * F3(*nt, i, j, k - 1) + w1[j] * F3(*nt, i, j + 1, k - 1) +
                                           w0[j] * F3(*nt, i, j, k) + w1[j] * F3(*nt, i, j + 1, k));
                double nu_z2 = nu + 0.5 * (w0[j] * F3(*nt, i, j, k) + w1[j] * F3(*nt, i, j + 1, k) +
                                           w0[j] * F3(*nt, i, j, k + 1) + w1[j] * F3(*nt, i, j + 1, k + 1));
                double visc =
                    1.0 / dx_3 * (nu_x2 * ((F3(*V, i + 1, j, k) - F3(*V, i, j, k)) / dx_2 + (F3(*U, i, j + 1, k) - F3(*U, i, j, k)) / dy_3) -
                                  nu_x1 * ((F3(*V, i, j, k) - F3(*V, i - 1, j, k)) / dx_1 + (F3(*U, i - 1, j + 1, k) - F3(*U, i - 1, j, k)) / dy_3)) +
                    2.0 / dy_3 * (nu_y2 * (F3(*V, i, j + 1, k) - F3(*V, i, j, k)) / dy_2 - nu_y1 * (F3(*V, i, j, k) - F3(*V, i, j - 1, k)) / dy_1) +
                    1.0 / dz_3 * (nu_z2 * ((F3(*V, i, j, k + 1) - F3(*V, i, j, k)) / dz_2 + (F3(*W, i, j + 1, k) - F3(*W, i, j, k)) / dy_3) -
                                  nu_z1 * ((F3(*V, i, j, k) - F3(*V, i, j, k - 1)) / dz_1 + (F3(*W, i, j + 1, k - 1) - F3(*W, i, j, k - 1)) / dy_3));
                r = r + visc;
                /* rotation (:334-342): term = interpolate_x(U,1) at centre i, then interpolate_y */
                if (fabs(Om) > 1e-6) {
                    double tu0 = 0.5 * (F3(*U, i - 1, j, k) + F3(*U, i, j, k));
                    double tu1 = 0.5 * (F3(*U, i - 1, j + 1, k) + F3(*U, i, j + 1, k));
                    r = r - 2.0 * Om * (w0[j] * tu0 + w1[j] * tu1);
                }
                F3(*R, i, j, k) = r;
            }
        }
    }
}

void cfo_compute_rhs_w(cfo *o, int slot) {
    /* equations.f90:351-498 */
    int nxg = o->nxg, nyg = o->nyg, nz = o->nz;
    fa *U = &o->U, *V = &o->V, *W = &o->W, *nt = &o->nu_t, *R = &o->Fw[slot];
    const double *x = o->x, *y = o->y, *z = o->z, *xg = o->xg, *yg = o->yg, *zg = o->zg;
    const double *w0 = o->weight_y_0, *w1 = o->weight_y_1;
    double nu = o->nu, dPdz = o->dPdz;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nz - 1; k++) {
        double dz_1 = z[k] - z[k - 1], dz_2 = z[k + 1] - z[k], dz_3 = zg[k + 1] - zg[k];
        for (int j = 2; j <= nyg - 1; j++) {
            double dy_3 = y[j] - y[j - 1];
            for (int i = 2; i <= nxg - 1; i++) {
                /* 1) -dw^2/dz (:370-384) */
                double a = 0.5 * (F3(*W, i, j, k) + F3(*W, i, j, k + 1));
                double b = 0.5 * (F3(*W, i, j, k - 1) + F3(*W, i, j, k));
                a = a * a; b = b * b;
                double r = -(a - b) / (zg[k + 1] - zg[k]);
                /* 2) -duw/dx (:389-406) */
                double uz1 = 0.5 * (F3(*U, i, j, k) + F3(*U, i, j, k + 1));
                double uz0 = 0.5 * (F3(*U, i - 1, j, k) + F3(*U, i - 1, j, k + 1));
                double wx1 = 0.5 * (F3(*W, i, j, k) + F3(*W, i + 1, j, k));
                double wx0 = 0.5 * (F3(*W, i - 1, j, k) + F3(*W, i, j, k));
                r = r + (-(uz1 * wx1 - uz0 * wx0) / (x[i] - x[i - 1]));
                /* 3) -dvw/dy (:411-428) */
                double vz1 = 0.5 * (F3(*V, i, j, k) + F3(*V, i, j, k + 1));
                double vz0 = 0.5 * (F3(*V, i, j - 1, k) + F3(*V, i, j - 1, k + 1));
                double wy1 = w0[j] * F3(*W, i, j, k) + w1[j] * F3(*W, i, j + 1, k);
                double wy0 = w0[j - 1] * F3(*W, i, j - 1, k) + w1[j - 1] * F3(*W, i, j, k);
                r = r + (-(vz1 * wy1 - vz0 * wy0) / (y[j] - y[j - 1]));
                /* 4) viscous (:435-493) */
                double dx_1 = xg[i] - xg[i - 1], dx_2 = xg[i + 1] - xg[i], dx_3 = x[i] - x[i - 1];
                double t2j = (F3(*W, i, j + 1, k) - F3(*W, i, j, k)) / (yg[j + 1] - yg[j]);
                double t2jm = (F3(*W, i, j, k) - F3(*W, i, j - 1, k)) / (yg[j] - yg[j - 1]);
                double nu_x1 = nu + 0.25 * (F3(*nt, i, j, k) + F3(*nt, i, j, k + 1) + F3(*nt, i - 1, j, k) + F3(*nt, i - 1, j, k + 1));
                double nu_x2 = nu + 0.25 * (F3(*nt, i, j, k) + F3(*nt, i, j, k + 1) + F3(*nt, i + 1, j, k) + F3(*nt, i + 1, j, k + 1));
                double nu_y1 = nu + 0.5 * (w0[j - 1] * F3(*nt, i, j - 1, k) + w1[j - 1] * F3(*nt, i, j, k) +
                                           w0[j - 1] * F3(*nt, i, j - 1, k + 1) + w1[j - 1] * F3(*nt, i, j, k + 1));
                double nu_y2 = nu + 0.5 * (w0[j] * F3(*nt, i, j, k) + w1[j] * F3(*nt, i, j + 1, k) +
                                           w0[j] * F3(*nt, i, j, k + 1) + w1[j] * F3(*nt, i, j + 1, k + 1));
                double nu_z1 = nu + F3(*nt, i, j, k);
                double nu_z2 = nu + F3(*nt, i, j, k + 1);
                double visc =
                    1.0 / dx_3 * (nu_x2 * ((F3(*W, i + 1, j, k) - F3(*W, i, j, k)) / dx_2 + (F3(*U, i, j, k + 1) - F3(*U, i, j, k)) / dz_2) -
                                  nu_x1 * ((F3(*W, i, j, k) - F3(*W, i - 1, j, k)) / dx_1 + (F3(*U, i - 1, j, k + 1) - F3(*U, i - 1, j, k)) / dz_1)) +
                    1.0 / dy_3 * (nu_y2 * (t2j + (F3(*V, i, j, k + 1) - F3(*V, i, j, k)) / dz_2) -
                                  nu_y1 * (t2jm + (F3(*V, i, j - 1, k + 1) - F3(*V, i, j - 1, k)) / dz_1)) +
                    2.0 / dz_3 * (nu_z2 * (F3(*W, i, j, k + 1) - F3(*W, i, j, k)) / dz_2 - nu_z1 * (F3(*W, i, j, k) - F3(*W, i, j, k - 1)) / dz_1);
                r = r + visc;
                r = r + dPdz; /* :496 */
                F3(*R, i, j, k) = r;
            }
        }
    }
}

/* RK3 stage update, time_integration.f90:108-110, 124-126, 140-145 */
void cfo_rk_update(cfo *o, int s) {
    double dt = o->dt;
    double (*c)[4] = o->rk_coef;
    int nx = o->nx, nxg = o->nxg, ny = o->ny, nyg = o->nyg, nz = o->nz, nzg = o->nzg;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nx - 1; i++) {
                double f;
                if (s == 1) f = dt * c[1][1] * F3(o->Fu[1], i, j, k);
                else if (s == 2) f = dt * (c[2][1] * F3(o->Fu[1], i, j, k) + c[2][2] * F3(o->Fu[2], i, j, k));
                else f = dt * (c[3][1] * F3(o->Fu[1], i, j, k) + c[3][2] * F3(o->Fu[2], i, j, k) + c[3][3] * F3(o->Fu[3], i, j, k));
                F3(o->U, i, j, k) = F3(o->Uo, i, j, k) + f;
            }
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= ny - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) {
                double f;
                if (s == 1) f = dt * c[1][1] * F3(o->Fv[1], i, j, k);
                else if (s == 2) f = dt * (c[2][1] * F3(o->Fv[1], i, j, k) + c[2][2] * F3(o->Fv[2], i, j, k));
                else f = dt * (c[3][1] * F3(o->Fv[1], i, j, k) + c[3][2] * F3(o->Fv[2], i, j, k) + c[3][3] * F3(o->Fv[3], i, j, k));
                F3(o->V, i, j, k) = F3(o->Vo, i, j, k) + f;
            }
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nz - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) {
                double f;
                if (s == 1) f = dt * c[1][1] * F3(o->Fw[1], i, j, k);
                else if (s == 2) f = dt * (c[2][1] * F3(o->Fw[1], i, j, k) + c[2][2] * F3(o->Fw[2], i, j, k));
                else f = dt * (c[3][1] * F3(o->Fw[1], i, j, k) + c[3][2] * F3(o->Fw[2], i, j, k) + c[3][3] * F3(o->Fw[3], i, j, k));
                F3(o->W, i, j, k) = F3(o->Wo, i, j, k) + f;
            }
}

/* ------------------------------------------------------------------------ */
/* Dynamic Smagorinsky, subgrid.f90:376-538 and helpers                      */
/* ------------------------------------------------------------------------ */
/* filter_xzy, subgrid.f90:140-187, applied to the section
 *   in(i0 : i0+n1-1, j0 : j0+n2-1, k0 : k0+n3-1, cin)
 * writing the result Uf_(1:n1-2, 1:n2, 1:n3-2) to out starting at (oi, oj, ok, cout).
 * Each output element accumulates its 9 (x,z) taps in the reference order. */
static void filter_xzy(const fa *in, int i0, int n1, int j0, int n2, int k0, int n3, int cin,
                       fa *out, int oi, int oj, int ok, int cout) {
    double fil[3][3];
    fil[0][0] = 1.0 / 36.0; fil[2][2] = 1.0 / 36.0; fil[0][2] = 1.0 / 36.0; fil[2][0] = 1.0 / 36.0;
    fil[1][2] = 1.0 / 9.0; fil[2][1] = 1.0 / 9.0; fil[1][0] = 1.0 / 9.0; fil[0][1] = 1.0 / 9.0;
    fil[1][1] = 4.0 / 9.0;
    const double c6 = 1.0 / 6.0, c23 = 2.0 / 3.0, c13 = 1.0 / 3.0;
#pragma omp parallel for schedule(static)
    for (int kk = 2; kk <= n3 - 1; kk++)
        for (int j = 1; j <= n2; j++)
            for (int ii = 2; ii <= n1 - 1; ii++) {
                double acc = 0.0;
                for (int a = -1; a <= 1; a++)
                    for (int c = -1; c <= 1; c++) {
                        int iA = i0 + ii + a - 1, kA = k0 + kk + c - 1, jA = j0 + j - 1;
                        double v;
                        if (j >= 2 && j <= n2 - 1)
                            v = c6 * F4(*in, iA, jA - 1, kA, cin) + c23 * F4(*in, iA, jA, kA, cin) + c6 * F4(*in, iA, jA + 1, kA, cin);
                        else if (j == 1)
                            v = c23 * F4(*in, iA, jA, kA, cin) + c13 * F4(*in, iA, jA + 1, kA, cin);
                        else
                            v = c13 * F4(*in, iA, jA - 1, kA, cin) + c23 * F4(*in, iA, jA, kA, cin);
                        acc = acc + v * fil[a + 1][c + 1];
                    }
                F4(*out, oi + ii - 2, oj + j - 1, ok + kk - 2, cout) = acc;
            }
}

/* compute_Sij, subgrid.f90:891-949 */
static void compute_Sij(cfo *o, fa *U, fa *V, fa *W, fa *Sij, fa *S) {
    int nxg = o->nxg, nyg = o->nyg, nzg = o->nzg;
    const double *x = o->x, *y = o->y, *z = o->z, *xg = o->xg, *yg = o->yg, *zg = o->zg;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) {
                F4(*Sij, i, j, k, 1) = (F3(*U, i, j, k) - F3(*U, i - 1, j, k)) / (x[i] - x[i - 1]);
                F4(*Sij, i, j, k, 2) = (F3(*V, i, j, k) - F3(*V, i, j - 1, k)) / (y[j] - y[j - 1]);
                F4(*Sij, i, j, k, 3) = (F3(*W, i, j, k) - F3(*W, i, j, k - 1)) / (z[k] - z[k - 1]);
            }
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg; k++)
        for (int j = 2; j <= nyg; j++)
            for (int i = 2; i <= nxg; i++) {
                F4(*Sij, i, j, k, 4) = 0.5 * ((F3(*U, i - 1, j, k) - F3(*U, i - 1, j - 1, k)) / (yg[j] - yg[j - 1]) +
                                              (F3(*V, i, j - 1, k) - F3(*V, i - 1, j - 1, k)) / (xg[i] - xg[i - 1]));
                F4(*Sij, i, j, k, 5) = 0.5 * ((F3(*U, i - 1, j, k) - F3(*U, i - 1, j, k - 1)) / (zg[k] - zg[k - 1]) +
                                              (F3(*W, i, j, k - 1) - F3(*W, i - 1, j, k - 1)) / (xg[i] - xg[i - 1]));
                F4(*Sij, i, j, k, 6) = 0.5 * ((F3(*V, i, j - 1, k) - F3(*V, i, j - 1, k - 1)) / (zg[k] - zg[k - 1]) +
                                              (F3(*W, i, j, k - 1) - F3(*W, i, j - 1, k - 1)) / (yg[j] - yg[j - 1]));
            }
    /* edge -> centre.  The reference updates in place in increasing (k,j,i)
     * order, and every update reads only entries it has not yet overwritten,
     * so computing into a temporary and copying back gives the same values. */
    fa *Sc = &o->Sc;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) {
                F4(*Sc, i, j, k, 1) = 0.25 * (F4(*Sij, i, j, k, 4) + F4(*Sij, i + 1, j, k, 4) + F4(*Sij, i, j + 1, k, 4) + F4(*Sij, i + 1, j + 1, k, 4));
                F4(*Sc, i, j, k, 2) = 0.25 * (F4(*Sij, i, j, k, 5) + F4(*Sij, i + 1, j, k, 5) + F4(*Sij, i, j, k + 1, 5) + F4(*Sij, i + 1, j, k + 1, 5));
                F4(*Sc, i, j, k, 3) = 0.25 * (F4(*Sij, i, j, k, 6) + F4(*Sij, i, j + 1, k, 6) + F4(*Sij, i, j, k + 1, 6) + F4(*Sij, i, j + 1, k + 1, 6));
            }
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                for (int c = 4; c <= 6; c++) F4(*Sij, i, j, k, c) = F4(*Sc, i, j, k, c - 3);
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) {
                double s = 0.0;
                for (int c = 1; c <= 6; c++) {
                    double v = F4(*Sij, i, j, k, c);
                    if (c <= 3) s = s + 2.0 * v * v;
                    else s = s + 4.0 * v * v;
                }
                F3(*S, i, j, k) = sqrt(s);
            }
}

static void sgs_dynamic_smagorinsky(cfo *o) {
    int nx = o->nx, nxg = o->nxg, ny = o->ny, nyg = o->nyg, nz = o->nz, nzg = o->nzg;
    fa *U = &o->U, *V = &o->V, *W = &o->W;
    fa *term = &o->term, *term_1 = &o->term_1, *term_2 = &o->term_2;
    fa *Sij = &o->Sij, *Lij = &o->Lij, *Mij = &o->Mij, *S = &o->S, *tb = &o->ten_buf;

    /* Part 1 (subgrid.f90:390-427): centre velocities */
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nzg; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 2; i <= nxg - 1; i++) F3(*term, i, j, k) = 0.5 * (F3(*U, i - 1, j, k) + F3(*U, i, j, k));
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nzg; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 1; i <= nxg; i++) F3(*term_1, i, j, k) = 0.5 * (F3(*V, i, j - 1, k) + F3(*V, i, j, k));
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 1; i <= nxg; i++)
                F3(*term_2, i, j, k) = (k <= nz) ? 0.5 * (F3(*W, i, j, k - 1) + F3(*W, i, j, k)) : 0.0;
    periodic_x(term, 2, nx, nxg, 1);
    periodic_z(term_2, 4, nz, nzg, 1);

    /* products u_i u_j at centres into Sij (placeholder), then ten_buf */
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg; i++) {
                double u = F3(*term, i, j, k), v = F3(*term_1, i, j, k), w = F3(*term_2, i, j, k);
                F4(*Sij, i, j, k, 1) = u * u;
                F4(*Sij, i, j, k, 2) = v * v;
                F4(*Sij, i, j, k, 3) = w * w;
                F4(*Sij, i, j, k, 4) = u * v;
                F4(*Sij, i, j, k, 5) = u * w;
                F4(*Sij, i, j, k, 6) = v * w;
                for (int c = 1; c <= 6; c++) F4(*tb, i, j, k, c) = F4(*Sij, i, j, k, c);
            }
    for (int c = 1; c <= 6; c++) {
        periodic_x(tb, 2, nx, nxg, c);
        periodic_z(tb, 4, nz, nzg, c);
    }
    /* Lij = hat(ui uj) on (2:nxg-1, 2:nyg-1, 2:nzg-1) */
    for (int c = 1; c <= 6; c++) filter_xzy(tb, 1, nxg, 2, nyg - 2, 1, nzg, c, Lij, 2, 2, 2, c);
    /* hat(ui) */
    filter_xzy(term, 1, nxg, 2, nyg - 2, 1, nzg, 1, Sij, 2, 2, 2, 1);
    filter_xzy(term_1, 1, nxg, 2, nyg - 2, 1, nzg, 1, Sij, 2, 2, 2, 2);
    filter_xzy(term_2, 1, nxg, 2, nyg - 2, 1, nzg, 1, Sij, 2, 2, 2, 3);
    /* Lij = hat(ui uj) - hat(ui) hat(uj) (only the interior is used later) */
    static const int ca[7] = {0, 1, 2, 3, 1, 1, 2}, cb[7] = {0, 1, 2, 3, 2, 3, 3};
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                for (int c = 1; c <= 6; c++)
                    F4(*Lij, i, j, k, c) = F4(*Lij, i, j, k, c) - F4(*Sij, i, j, k, ca[c]) * F4(*Sij, i, j, k, cb[c]);

    /* Part 2 (subgrid.f90:429-482): filtered velocities */
    filter_xzy(U, 1, nx, 1, nyg, 1, nzg, 1, &o->Uf, 2, 1, 2, 1);
    filter_xzy(V, 1, nxg, 1, ny, 1, nzg, 1, &o->Vf, 2, 1, 2, 1);
    filter_xzy(W, 1, nxg, 1, nyg, 1, nz, 1, &o->Wf, 2, 1, 2, 1);
    periodic_x(&o->Uf, 1, nx, nxg, 1);
    periodic_z(&o->Uf, 1, nz, nzg, 1);
    periodic_x(&o->Vf, 2, nx, nxg, 1);
    periodic_z(&o->Vf, 2, nz, nzg, 1);
    periodic_x(&o->Wf, 2, nx, nxg, 1);
    periodic_z(&o->Wf, 3, nz, nzg, 1);

    compute_Sij(o, &o->Uf, &o->Vf, &o->Wf, Sij, S);
    o->fil_size = 2.0; /* set inside filter_xzy, subgrid.f90:156 */
    double fs2 = pow(o->fil_size, 2.0);
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                for (int c = 1; c <= 6; c++) F4(*Mij, i, j, k, c) = fs2 * F3(*S, i, j, k) * F4(*Sij, i, j, k, c);

    compute_Sij(o, U, V, W, Sij, S);
    for (int c = 1; c <= 6; c++) {
#pragma omp parallel for schedule(static)
        for (int k = 2; k <= nzg - 1; k++)
            for (int j = 2; j <= nyg - 1; j++)
                for (int i = 2; i <= nxg - 1; i++) F3(*term, i, j, k) = F3(*S, i, j, k) * F4(*Sij, i, j, k, c);
        periodic_x(term, 2, nx, nxg, 1);
        periodic_z(term, 4, nz, nzg, 1);
        filter_xzy(term, 1, nxg, 2, nyg - 2, 1, nzg, 1, Sij, 2, 2, 2, c);
    }
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                for (int c = 1; c <= 6; c++) F4(*Mij, i, j, k, c) = F4(*Mij, i, j, k, c) - F4(*Sij, i, j, k, c);

    /* Part 3 (subgrid.f90:484-536) */
    fa *nt = &o->nu_t;
    for (size_t q = 0; q < fa_size(nt); q++) nt->p[q] = 0.0;
    double *LMk = (double *)calloc((size_t)(nyg + 1) * (nzg + 1), sizeof(double));
    double *MMk = (double *)calloc((size_t)(nyg + 1) * (nzg + 1), sizeof(double));
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++) {
            double sl = 0.0, sm = 0.0;
            for (int i = 2; i <= nxg - 1; i++) {
                double lm = (F4(*Lij, i, j, k, 1) * F4(*Mij, i, j, k, 1) + F4(*Lij, i, j, k, 2) * F4(*Mij, i, j, k, 2) +
                             F4(*Lij, i, j, k, 3) * F4(*Mij, i, j, k, 3) +
                             2.0 * (F4(*Lij, i, j, k, 4) * F4(*Mij, i, j, k, 4) + F4(*Lij, i, j, k, 5) * F4(*Mij, i, j, k, 5) +
                                    F4(*Lij, i, j, k, 6) * F4(*Mij, i, j, k, 6)));
                double mm = (F4(*Mij, i, j, k, 1) * F4(*Mij, i, j, k, 1) + F4(*Mij, i, j, k, 2) * F4(*Mij, i, j, k, 2) +
                             F4(*Mij, i, j, k, 3) * F4(*Mij, i, j, k, 3) +
                             2.0 * (F4(*Mij, i, j, k, 4) * F4(*Mij, i, j, k, 4) + F4(*Mij, i, j, k, 5) * F4(*Mij, i, j, k, 5) +
                                    F4(*Mij, i, j, k, 6) * F4(*Mij, i, j, k, 6)));
                sl += lm;
                sm += mm;
            }
            LMk[(size_t)j * (nzg + 1) + k] = sl;
            MMk[(size_t)j * (nzg + 1) + k] = sm;
        }
    for (int j = 2; j <= nyg - 1; j++) {
        double sl = 0.0, sm = 0.0;
        for (int k = 2; k <= nzg - 1; k++) { sl += LMk[(size_t)j * (nzg + 1) + k]; sm += MMk[(size_t)j * (nzg + 1) + k]; }
        F3(o->avg_nu_t, 1, j, 1) = sl / sm;
    }
    free(LMk); free(MMk);
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) F3(*nt, i, j, k) = -0.5 * F3(o->avg_nu_t, 1, j, 1) * F3(*S, i, j, k);
    periodic_x(nt, 2, nx, nxg, 1);
    periodic_z(nt, 4, nz, nzg, 1);
    /* clipping (NaN -> 0) */
    for (size_t q = 0; q < fa_size(nt); q++) nt->p[q] = (nt->p[q] > 0.0) ? nt->p[q] : 0.0;
    if (o->p.Dirichlet_nu_t == 1) {
        dirichlet_y(nt, 2, ny, nyg);
        F3(o->avg_nu_t, 1, 1, 1) = -F3(o->avg_nu_t, 1, 2, 1);
        F3(o->avg_nu_t, 1, nyg, 1) = -F3(o->avg_nu_t, 1, nyg - 1, 1);
    } else {
        neumann_y(nt, 2, ny, nyg);
        F3(o->avg_nu_t, 1, 1, 1) = F3(o->avg_nu_t, 1, 2, 1);
        F3(o->avg_nu_t, 1, nyg, 1) = F3(o->avg_nu_t, 1, nyg - 1, 1);
    }
}

/* ------------------------------------------------------------------------ */
/* Anisotropic minimum dissipation model, subgrid.f90:639-881.               */
/* The reference works on whole arrays and array sections of the module     */
/* temporaries term, term_1..term_4, some of which it only partly sets; the */
/* restatement performs the same section operations on temporaries filled  */
/* with NaN, so a value the reference would take from an unset (stale)      */
/* part of a temporary shows as NaN.  amd_nan_canonical counts the          */
/* canonical cells whose quotient came out NaN.                             */
/* ------------------------------------------------------------------------ */
typedef struct { int l[3], u[3]; } sec3;
static sec3 SEC(int l0, int u0, int l1, int u1, int l2, int u2) {
    sec3 r = {{l0, l1, l2}, {u0, u1, u2}};
    return r;
}
/* interpolate_x/_y/_z(u = A(a), ui = B(b), 1), interpolation.f90:24-105:
 * ui = 0, then ui(1:n-1 along dir) = 0.5 (u(m) + u(m+1)) with n = shape(u). */
static void interp_sec(int dir, fa *A, sec3 a, fa *B, sec3 b) {
    int m[3];
    for (int d = 0; d < 3; d++) m[d] = a.u[d] - a.l[d] + 1;
    m[dir] -= 1;
    for (int d = 0; d < 3; d++)
        if (b.l[d] + m[d] - 1 > b.u[d]) {
            fprintf(stderr, "cf_oracle: interpolation section overflow\n");
            abort();
        }
    for (int k = b.l[2]; k <= b.u[2]; k++)
        for (int j = b.l[1]; j <= b.u[1]; j++)
            for (int i = b.l[0]; i <= b.u[0]; i++) F3(*B, i, j, k) = 0.0;
    for (int r = 0; r < m[2]; r++)
        for (int q = 0; q < m[1]; q++)
            for (int p = 0; p < m[0]; p++) {
                int e[3] = {p, q, r};
                e[dir] += 1;
                F3(*B, b.l[0] + p, b.l[1] + q, b.l[2] + r) =
                    0.5 * (F3(*A, a.l[0] + p, a.l[1] + q, a.l[2] + r) + F3(*A, a.l[0] + e[0], a.l[1] + e[1], a.l[2] + e[2]));
            }
}
#define AMD_LOOP(i0, i1, j0, j1, k0, k1) \
    for (int k = (k0); k <= (k1); k++)    \
        for (int j = (j0); j <= (j1); j++) \
            for (int i = (i0); i <= (i1); i++)
static double sq(double a) { return pow(a, 2.0); }

static void sgs_amd(cfo *o) {
    int nx = o->nx, ny = o->ny, nz = o->nz, nxg = o->nxg, nyg = o->nyg, nzg = o->nzg;
    const double *x = o->x, *y = o->y, *z = o->z, *xg = o->xg, *yg = o->yg, *zg = o->zg;
    fa *U = &o->U, *V = &o->V, *W = &o->W, *Sij = &o->Sij, *nt = &o->nu_t;
    const double C = 0.3;
    fa t0 = fa_new3(1, nxg, 1, nyg, 1, nzg), t1 = fa_new3(1, nxg, 1, nyg, 1, nzg), t2 = fa_new3(1, nxg, 1, nyg, 1, nzg);
    fa t3 = fa_new3(1, nxg, 1, nyg, 1, nzg), t4 = fa_new3(1, nxg, 1, nyg, 1, nzg);
    fa *tt[5] = {&t0, &t1, &t2, &t3, &t4};
    for (int q = 0; q < 5; q++)
        for (size_t e = 0; e < fa_size(tt[q]); e++) tt[q]->p[e] = NAN;
    const sec3 ALL = SEC(1, nxg, 1, nyg, 1, nzg);
    /* Part 1: subgrid.f90:658 */
    compute_Sij(o, U, V, W, Sij, &o->S);
    /* nu += f * T(2:nxg,2:nyg,2:nzg) * Sij(:,:,:,c) */
#define NU_ADD(f, T, c) AMD_LOOP(2, nxg, 2, nyg, 2, nzg) F3(*nt, i, j, k) = F3(*nt, i, j, k) + (f) * F3(T, i, j, k) * F4(*Sij, i, j, k, c)
#define NU_ADD1(T, c) AMD_LOOP(2, nxg, 2, nyg, 2, nzg) F3(*nt, i, j, k) = F3(*nt, i, j, k) + F3(T, i, j, k) * F4(*Sij, i, j, k, c)
#define WHOLE(stmt) AMD_LOOP(ALL.l[0], ALL.u[0], ALL.l[1], ALL.u[1], ALL.l[2], ALL.u[2]) stmt

    /* (d_hat_i U)^2 S11, (d_i U)^2: subgrid.f90:660-695 */
    for (int i = 2; i <= nx; i++)
        for (int k = 1; k <= nzg; k++)
            for (int j = 1; j <= nyg; j++) {
                F3(t2, i, j, k) = sq(F3(*U, i, j, k) - F3(*U, i - 1, j, k));
                F3(t4, i, j, k) = sq(F3(*U, i, j, k) - F3(*U, i - 1, j, k)) / sq(x[i] - x[i - 1]);
            }
    AMD_LOOP(2, nxg, 2, nyg, 2, nzg) F3(*nt, i, j, k) = F3(t2, i, j, k) * F4(*Sij, i, j, k, 1);
    for (int j = 2; j <= nyg; j++)
        for (int k = 1; k <= nzg; k++)
            for (int i = 1; i <= nx; i++) {
                F3(t0, i, j, k) = sq(F3(*U, i, j, k) - F3(*U, i, j - 1, k));
                F3(t1, i, j, k) = F3(t0, i, j, k) / sq(yg[j] - yg[j - 1]);
            }
    interp_sec(0, &t1, SEC(1, nx, 2, nyg, 1, nzg), &t2, SEC(2, nx, 2, nyg, 1, nzg));
    interp_sec(1, &t2, SEC(2, nx, 2, nyg, 1, nzg), &t3, SEC(2, nx, 2, nyg - 1, 1, nzg));
    WHOLE(F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t3, i, j, k));
    interp_sec(0, &t0, SEC(1, nx, 2, nyg, 1, nzg), &t1, SEC(2, nx, 2, nyg, 1, nzg));
    interp_sec(1, &t1, SEC(2, nx, 2, nyg, 1, nzg), &t2, SEC(2, nx, 2, nyg - 1, 1, nzg));
    NU_ADD1(t2, 1);
    for (int k = 2; k <= nzg; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 1; i <= nx; i++) {
                F3(t0, i, j, k) = sq(F3(*U, i, j, k) - F3(*U, i, j, k - 1));
                F3(t1, i, j, k) = F3(t0, i, j, k) / sq(zg[k] - zg[k - 1]);
            }
    interp_sec(0, &t1, SEC(1, nx, 1, nyg, 2, nzg), &t2, SEC(2, nx, 1, nyg, 2, nzg));
    interp_sec(2, &t2, SEC(2, nx, 1, nyg, 2, nzg), &t3, SEC(2, nx, 1, nyg, 2, nzg - 1));
    WHOLE(F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t3, i, j, k));
    interp_sec(0, &t0, SEC(1, nx, 1, nyg, 2, nzg), &t1, SEC(2, nx, 1, nyg, 2, nzg));
    interp_sec(2, &t1, SEC(2, nx, 1, nyg, 2, nzg), &t2, SEC(2, nx, 1, nyg, 2, nzg - 1));
    NU_ADD1(t2, 1);

    /* (d_hat_i V)^2 S22, (d_i V)^2: subgrid.f90:697-731 */
    for (int j = 2; j <= ny; j++)
        for (int k = 1; k <= nzg; k++)
            for (int i = 1; i <= nxg; i++) {
                F3(t2, i, j, k) = sq(F3(*V, i, j, k) - F3(*V, i, j - 1, k));
                F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t2, i, j, k) / sq(y[j] - y[j - 1]);
            }
    NU_ADD1(t2, 2);
    for (int i = 2; i <= nxg; i++)
        for (int k = 1; k <= nzg; k++)
            for (int j = 1; j <= ny; j++) {
                F3(t0, i, j, k) = sq(F3(*V, i, j, k) - F3(*V, i - 1, j, k));
                F3(t1, i, j, k) = F3(t0, i, j, k) / sq(xg[i] - xg[i - 1]);
            }
    interp_sec(1, &t1, SEC(2, nxg, 1, ny, 1, nzg), &t2, SEC(2, nxg, 2, ny, 1, nzg));
    interp_sec(0, &t2, SEC(2, nxg, 2, ny, 1, nzg), &t3, SEC(2, nxg - 1, 2, ny, 1, nzg));
    WHOLE(F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t3, i, j, k));
    interp_sec(1, &t0, SEC(2, nxg, 1, ny, 1, nzg), &t1, SEC(2, nxg, 2, ny, 1, nzg));
    interp_sec(0, &t1, SEC(2, nxg, 2, ny, 1, nzg), &t2, SEC(2, nxg - 1, 2, ny, 1, nzg));
    NU_ADD1(t2, 2);
    for (int k = 2; k <= nzg; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nxg; i++) {
                F3(t0, i, j, k) = sq(F3(*V, i, j, k) - F3(*V, i, j, k - 1));
                F3(t1, i, j, k) = F3(t0, i, j, k) / sq(zg[k] - zg[k - 1]);
            }
    interp_sec(1, &t1, SEC(1, nxg, 1, ny, 2, nzg), &t2, SEC(1, nxg, 2, ny, 2, nzg));
    interp_sec(2, &t2, SEC(1, nxg, 2, ny, 2, nzg), &t3, SEC(1, nxg, 2, ny, 2, nzg - 1));
    WHOLE(F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t3, i, j, k));
    interp_sec(1, &t0, SEC(1, nxg, 1, ny, 2, nzg), &t1, SEC(1, nxg, 2, ny, 2, nzg));
    interp_sec(2, &t1, SEC(1, nxg, 2, ny, 2, nzg), &t2, SEC(1, nxg, 2, ny, 2, nzg - 1));
    NU_ADD1(t2, 2);

    /* (d_hat_i W)^2 S33, (d_i W)^2: subgrid.f90:733-767 */
    for (int k = 2; k <= nz; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 1; i <= nxg; i++) {
                F3(t2, i, j, k) = sq(F3(*W, i, j, k) - F3(*W, i, j, k - 1));
                F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t2, i, j, k) / sq(z[k] - z[k - 1]);
            }
    NU_ADD1(t2, 3);
    for (int i = 2; i <= nxg; i++)
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= nyg; j++) {
                F3(t0, i, j, k) = sq(F3(*W, i, j, k) - F3(*W, i - 1, j, k));
                F3(t1, i, j, k) = F3(t0, i, j, k) / sq(xg[i] - xg[i - 1]);
            }
    interp_sec(2, &t1, SEC(2, nxg, 1, nyg, 1, nz), &t2, SEC(2, nxg, 1, nyg, 2, nz));
    interp_sec(0, &t2, SEC(2, nxg, 1, nyg, 2, nz), &t3, SEC(2, nxg - 1, 1, nyg, 2, nz));
    WHOLE(F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t3, i, j, k));
    interp_sec(2, &t0, SEC(2, nxg, 1, nyg, 1, nz), &t1, SEC(2, nxg, 1, nyg, 2, nz));
    interp_sec(0, &t1, SEC(2, nxg, 1, nyg, 2, nz), &t2, SEC(2, nxg - 1, 1, nyg, 2, nz));
    NU_ADD1(t2, 3);
    for (int j = 2; j <= nyg; j++)
        for (int k = 1; k <= nz; k++)
            for (int i = 1; i <= nxg; i++) {
                F3(t0, i, j, k) = sq(F3(*W, i, j, k) - F3(*W, i, j - 1, k));
                F3(t1, i, j, k) = F3(t0, i, j, k) / sq(yg[j] - yg[j - 1]);
            }
    interp_sec(2, &t1, SEC(1, nxg, 2, nyg, 1, nz), &t2, SEC(1, nxg, 2, nyg, 2, nz));
    interp_sec(1, &t2, SEC(1, nxg, 2, nyg, 2, nz), &t3, SEC(1, nxg, 2, nyg - 1, 2, nz));
    WHOLE(F3(t4, i, j, k) = F3(t4, i, j, k) + F3(t3, i, j, k));
    interp_sec(2, &t0, SEC(1, nxg, 2, nyg, 1, nz), &t1, SEC(1, nxg, 2, nyg, 2, nz));
    interp_sec(1, &t1, SEC(1, nxg, 2, nyg, 2, nz), &t2, SEC(1, nxg, 2, nyg - 1, 2, nz));
    NU_ADD1(t2, 3);

    /* 2 (d_hat_i U)(d_hat_i V) S12: subgrid.f90:769-800 */
    for (int i = 2; i <= nxg; i++)
        for (int k = 1; k <= nzg; k++)
            for (int j = 1; j <= ny; j++) F3(t0, i, j, k) = F3(*V, i, j, k) - F3(*V, i - 1, j, k);
    interp_sec(1, &t0, SEC(2, nxg, 1, ny, 1, nzg), &t1, SEC(2, nxg, 2, ny, 1, nzg));
    interp_sec(0, &t1, SEC(2, nxg, 2, ny, 1, nzg), &t2, SEC(2, nxg - 1, 2, ny, 1, nzg));
    for (int i = 2; i <= nx; i++)
        for (int k = 1; k <= nzg; k++)
            for (int j = 2; j <= nyg - 1; j++)
                F3(t1, i, j, k) = F3(t2, i, j, k) * (F3(*U, i, j, k) - F3(*U, i - 1, j, k));
    NU_ADD(2.0, t1, 4);
    for (int j = 2; j <= nyg; j++)
        for (int k = 1; k <= nzg; k++)
            for (int i = 1; i <= nx; i++) F3(t0, i, j, k) = F3(*U, i, j, k) - F3(*U, i, j - 1, k);
    interp_sec(0, &t0, SEC(1, nx, 2, nyg, 1, nzg), &t1, SEC(2, nx, 2, nyg, 1, nzg));
    interp_sec(1, &t1, SEC(2, nx, 2, nyg, 1, nzg), &t2, SEC(2, nx, 2, nyg - 1, 1, nzg));
    for (int j = 2; j <= ny; j++)
        for (int k = 1; k <= nzg; k++)
            for (int i = 2; i <= nxg - 1; i++)
                F3(t1, i, j, k) = F3(t2, i, j, k) * (F3(*V, i, j, k) - F3(*V, i, j - 1, k));
    NU_ADD(2.0, t1, 4);
    for (int k = 2; k <= nzg; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 1; i <= nx; i++) F3(t0, i, j, k) = F3(*U, i, j, k) - F3(*U, i, j, k - 1);
    interp_sec(0, &t0, SEC(1, nx, 1, nyg, 2, nzg), &t1, SEC(2, nx, 1, nyg, 2, nzg));
    for (int k = 2; k <= nzg; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nxg; i++) F3(t0, i, j, k) = F3(*V, i, j, k) - F3(*V, i, j, k - 1);
    interp_sec(1, &t0, SEC(1, nxg, 1, ny, 2, nzg), &t2, SEC(1, nxg, 2, ny, 2, nzg));
    WHOLE(F3(t3, i, j, k) = F3(t1, i, j, k) * F3(t2, i, j, k));
    interp_sec(2, &t3, SEC(2, nxg - 1, 2, nyg - 1, 2, nzg), &t1, SEC(2, nxg - 1, 2, nyg - 1, 2, nzg - 1));
    NU_ADD(2.0, t1, 4);

    /* 2 (d_hat_i U)(d_hat_i W) S13: subgrid.f90:802-833 */
    for (int i = 2; i <= nxg; i++)
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= nyg; j++) F3(t0, i, j, k) = F3(*W, i, j, k) - F3(*W, i - 1, j, k);
    interp_sec(2, &t0, SEC(2, nxg, 1, nyg, 1, nz), &t1, SEC(2, nxg, 1, nyg, 2, nz));
    interp_sec(0, &t1, SEC(2, nxg, 1, nyg, 2, nz), &t2, SEC(2, nxg - 1, 1, nyg, 2, nz));
    for (int i = 2; i <= nx; i++)
        for (int k = 1; k <= nzg; k++)
            for (int j = 2; j <= nyg - 1; j++)
                F3(t1, i, j, k) = F3(t2, i, j, k) * (F3(*U, i, j, k) - F3(*U, i - 1, j, k));
    NU_ADD(2.0, t1, 5);
    for (int k = 2; k <= nzg; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 1; i <= nx; i++) F3(t0, i, j, k) = F3(*U, i, j, k) - F3(*U, i, j, k - 1);
    interp_sec(0, &t0, SEC(1, nx, 1, nyg, 2, nzg), &t1, SEC(2, nx, 1, nyg, 2, nzg));
    interp_sec(2, &t1, SEC(2, nx, 1, nyg, 2, nzg), &t2, SEC(2, nx, 1, nyg, 2, nzg - 1));
    for (int k = 2; k <= nz; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 2; i <= nxg - 1; i++)
                F3(t1, i, j, k) = F3(t2, i, j, k) * (F3(*W, i, j, k) - F3(*W, i, j, k - 1));
    NU_ADD(2.0, t1, 5);
    for (int j = 2; j <= nyg; j++)
        for (int k = 1; k <= nzg; k++)
            for (int i = 1; i <= nx; i++) F3(t0, i, j, k) = F3(*U, i, j, k) - F3(*U, i, j - 1, k);
    interp_sec(0, &t0, SEC(1, nx, 2, nyg, 1, nzg), &t1, SEC(2, nx, 2, nyg, 1, nzg));
    for (int j = 2; j <= nyg; j++)
        for (int k = 1; k <= nz; k++)
            for (int i = 1; i <= nxg; i++) F3(t0, i, j, k) = F3(*W, i, j, k) - F3(*W, i, j - 1, k);
    interp_sec(2, &t0, SEC(1, nxg, 2, nyg, 1, nz), &t2, SEC(1, nxg, 2, nyg, 2, nz));
    WHOLE(F3(t3, i, j, k) = F3(t1, i, j, k) * F3(t2, i, j, k));
    interp_sec(1, &t3, SEC(2, nxg - 1, 2, nyg, 2, nzg - 1), &t1, SEC(2, nxg - 1, 2, nyg - 1, 2, nzg - 1));
    NU_ADD(2.0, t1, 5);

    /* 2 (d_hat_i V)(d_hat_i W) S23: subgrid.f90:835-866 */
    for (int j = 2; j <= nyg; j++)
        for (int k = 1; k <= nz; k++)
            for (int i = 1; i <= nxg; i++) F3(t0, i, j, k) = F3(*W, i, j, k) - F3(*W, i, j - 1, k);
    interp_sec(2, &t0, SEC(1, nxg, 2, nyg, 1, nz), &t1, SEC(1, nxg, 2, nyg, 2, nz));
    interp_sec(1, &t1, SEC(1, nxg, 2, nyg, 2, nz), &t2, SEC(1, nxg, 2, nyg - 1, 2, nz));
    for (int j = 2; j <= ny; j++)
        for (int k = 1; k <= nzg; k++)
            for (int i = 2; i <= nxg - 1; i++)
                F3(t1, i, j, k) = F3(t2, i, j, k) * (F3(*V, i, j, k) - F3(*V, i, j - 1, k));
    NU_ADD(2.0, t1, 6);
    for (int k = 2; k <= nzg; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nxg; i++) F3(t0, i, j, k) = F3(*V, i, j, k) - F3(*V, i, j, k - 1);
    interp_sec(1, &t0, SEC(1, nxg, 1, ny, 2, nzg), &t1, SEC(1, nxg, 2, ny, 2, nzg));
    interp_sec(2, &t1, SEC(1, nxg, 2, ny, 2, nzg), &t2, SEC(1, nxg, 2, ny, 2, nzg - 1));
    for (int k = 2; k <= nz; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 1; i <= nxg; i++)
                F3(t1, i, j, k) = F3(t2, i, j, k) * (F3(*W, i, j, k) - F3(*W, i, j, k - 1));
    NU_ADD(2.0, t1, 6);
    for (int i = 2; i <= nxg; i++)
        for (int k = 1; k <= nzg; k++)
            for (int j = 1; j <= ny; j++) F3(t0, i, j, k) = F3(*V, i, j, k) - F3(*V, i - 1, j, k);
    interp_sec(1, &t0, SEC(2, nxg, 1, ny, 1, nzg), &t1, SEC(2, nxg, 2, ny, 1, nzg));
    for (int i = 2; i <= nxg; i++)
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= nyg; j++) F3(t0, i, j, k) = F3(*W, i, j, k) - F3(*W, i - 1, j, k);
    interp_sec(2, &t0, SEC(2, nxg, 1, nyg, 1, nz), &t2, SEC(2, nxg, 1, nyg, 2, nz));
    WHOLE(F3(t3, i, j, k) = F3(t1, i, j, k) * F3(t2, i, j, k));
    interp_sec(0, &t3, SEC(2, nxg, 2, nyg - 1, 2, nzg - 1), &t1, SEC(2, nxg - 1, 2, nyg - 1, 2, nzg - 1));
    NU_ADD(2.0, t1, 6);
#undef NU_ADD
#undef NU_ADD1
#undef WHOLE

    /* quotient and clipping (NaN -> 0), subgrid.f90:868-871 */
    int nan_can = 0;
    for (int k = 1; k <= nzg; k++)
        for (int j = 1; j <= nyg; j++)
            for (int i = 1; i <= nxg; i++) {
                double v = -C * F3(*nt, i, j, k) / F3(t4, i, j, k);
                if (v != v && i >= 2 && i <= nxg - 2 && j >= 2 && j <= nyg - 1 && k >= 2 && k <= nzg - 2) nan_can++;
                F3(*nt, i, j, k) = v > 0.0 ? v : 0.0;
            }
    o->amd_nan_canonical = nan_can;
    /* subgrid.f90:873-876 (one slab: the interior-plane update is the wrap) */
    periodic_x(nt, 2, nx, nxg, 1);
    periodic_z(nt, 4, nz, nzg, 1);
    if (o->p.Dirichlet_nu_t == 1) {
        dirichlet_y(nt, 2, ny, nyg);
    } else if (o->p.Dirichlet_nu_t == 0) {
        neumann_y(nt, 2, ny, nyg);
    } else if (o->p.Dirichlet_nu_t == 2) {
        double g = 2.0 * 0.38 * pow(o->dPdx, 0.5) * (y[2] - y[1]) / 2.0;
        for (int k = 1; k <= nzg; k++)
            for (int i = 1; i <= nxg; i++) {
                F3(*nt, i, 1, k) = -F3(*nt, i, 2, k) + g;
                F3(*nt, i, nyg, k) = -F3(*nt, i, nyg - 1, k) + g;
            }
    }
    /* subgrid.f90:877-879: rows 1 and nyg of avg_nu_t are left as they were */
    for (int j = 2; j <= nyg - 1; j++) {
        double s = 0.0;
        for (int k = 2; k <= nzg - 2; k++)
            for (int i = 2; i <= nxg - 2; i++) s += F3(*nt, i, j, k);
        F3(o->avg_nu_t, 1, j, 1) = s / (double)((nxg - 3) * (nzg - 3));
    }
    for (int q = 0; q < 5; q++) fa_free(tt[q]);
}
#undef AMD_LOOP

void cfo_compute_eddy_viscosity(cfo *o) {
    /* subgrid.f90:23-47 */
    if (o->p.LES_model == 2) {
        sgs_dynamic_smagorinsky(o);
    } else if (o->p.LES_model == 3) {
        sgs_amd(o);
    } else if (o->p.LES_model == 0) {
        for (size_t q = 0; q < fa_size(&o->nu_t); q++) o->nu_t.p[q] = 0.0;
        for (size_t q = 0; q < fa_size(&o->avg_nu_t); q++) o->avg_nu_t.p[q] = 0.0;
    } else {
        fprintf(stderr, "cf_oracle: LES_model %d not restated\n", o->p.LES_model);
        abort();
    }
}

/* ------------------------------------------------------------------------ */
/* Equilibrium wall model: eqwm.f90 and wallmodel.f90:591-685, 1342-1378     */
/* ------------------------------------------------------------------------ */
/* eqwm.f90:20-50.  y_cv(ncv+1) is never set by the reference; the maximum is
 * taken over the ncv defined centroids. */
static void eqwm_grid(int ncv, double stretch, double h_wm, double *y_cv, double *y_fa) {
    int nfa = ncv + 1;
    y_fa[1] = 0.0;
    double inc = 1.0;
    for (int ifa = 2; ifa <= nfa; ifa++) {
        y_fa[ifa] = y_fa[ifa - 1] + inc;
        y_cv[ifa - 1] = 0.5 * (y_fa[ifa] + y_fa[ifa - 1]);
        inc = inc * stretch;
    }
    double y_max = y_cv[1];
    for (int icv = 1; icv <= ncv; icv++) if (y_cv[icv] > y_max) y_max = y_cv[icv];
    for (int ifa = 1; ifa <= nfa; ifa++) y_fa[ifa] = y_fa[ifa] / y_max * h_wm;
    for (int icv = 1; icv <= ncv; icv++) y_cv[icv] = y_cv[icv] / y_max * h_wm;
}

/* eqwm.f90:52-88 */
static void thomas(int n, const double *a, const double *b, const double *c, const double *d, double *x, double *cp, double *dp) {
    cp[1] = c[1] / b[1];
    dp[1] = d[1] / b[1];
    for (int i = 2; i <= n; i++) {
        double m = b[i] - cp[i - 1] * a[i];
        cp[i] = c[i] / m;
        dp[i] = (d[i] - dp[i - 1] * a[i]) / m;
    }
    x[n] = dp[n];
    for (int j = n - 1; j >= 1; j--) x[j] = dp[j] - cp[j] * x[j + 1];
}

/* eqwm.f90:90-223 */
static double solve_u_eqwm(double umag_les, double mu_lam, double rho_eq, double h_wm, int ncv, double stretch,
                           int *iter_out, double tau_wall_in) {
    const double kappa = 0.41, Aplus = 17.0, tol = 0.0000001, max_iter = 100;
    double tau_wall_lam = mu_lam * umag_les / h_wm;
    double *y_cv = vec1(ncv + 1), *y_fa = vec1(ncv + 1), *mu_fa = vec1(ncv + 1);
    double *b = vec1(ncv), *aa = vec1(ncv), *bb = vec1(ncv), *cc = vec1(ncv), *u = vec1(ncv), *cp = vec1(ncv), *dp = vec1(ncv);
    eqwm_grid(ncv, stretch, h_wm, y_cv, y_fa);
    int nfa = ncv + 1, iter = 0, done = 0;
    double tau_wall = tau_wall_in;
    while (done == 0) {
        double tau_wall_prev = tau_wall;
        for (int i = 1; i <= nfa; i++) mu_fa[i] = mu_lam * 1.0;
        for (int ifa = 2; ifa <= nfa; ifa++) {
            double nu_eq = mu_lam / rho_eq;
            double utau_eq = sqrt(tau_wall / rho_eq);
            double D = 1.0 - exp(-1.0 * y_fa[ifa] * utau_eq / nu_eq / Aplus);
            D = D * D;
            double mut = rho_eq * kappa * y_fa[ifa] * utau_eq * D;
            mu_fa[ifa] = mu_fa[ifa] + mut;
        }
        /* tridiagonal rows of A (eqwm.f90:152-193) */
        bb[ncv] = 1.0; aa[ncv] = 0.0; cc[ncv] = 0.0; b[ncv] = umag_les;
        for (int icv = 2; icv <= ncv - 1; icv++) {
            double sup = mu_fa[icv + 1] / (y_cv[icv + 1] - y_cv[icv]);
            double sub = mu_fa[icv] / (y_cv[icv] - y_cv[icv - 1]);
            bb[icv] = -1.0 * (sup + sub);
            cc[icv] = sup;
            aa[icv] = sub;
            b[icv] = 0.0;
        }
        b[1] = 0.0;
        double sup = mu_fa[2] / (y_cv[2] - y_cv[1]);
        bb[1] = -1.0 * (sup + mu_fa[1] / (y_cv[1] - y_fa[1]));
        cc[1] = sup;
        aa[1] = 0.0;
        thomas(ncv, aa, bb, cc, b, u, cp, dp);
        tau_wall = mu_fa[1] * (u[1] - 0.0) / (y_cv[1] - y_fa[1]);
        if (fabs((tau_wall - tau_wall_prev) / tau_wall_lam) < tol) done = 1;
        if (done == 0) iter = iter + 1;
        if (iter > max_iter) done = 1;
    }
    free(y_cv); free(y_fa); free(mu_fa); free(b); free(aa); free(bb); free(cc); free(u); free(cp); free(dp);
    *iter_out = iter;
    return tau_wall;
}

double cfo_solve_u_eqwm(double umag_les, double nu, double h_wm, int ncv, double stretch, double tau_in, int *iter) {
    /* one wall point of wallmodel.f90:621 (rho = 1) */
    return solve_u_eqwm(umag_les, nu, 1.0, h_wm, ncv, stretch, iter, tau_in);
}

/* interpolate_z_2nd (interpolation.f90:188-252) for u(1:n1,1,1:ny) -> ui(1:n1,1,1:n3) */
static void interp_z_2nd(const double *y, int ny, const fa *u, const double *yi, int n3, fa *ui) {
    int n1 = (int)u->n[0];
    int jj = 2;
    for (int j = 2; j <= n3 - 1; j++) {
        double yref = yi[j];
        for (int j2 = 3; j2 <= ny; j2++) if (y[j2] > yref) { jj = j2 - 1; break; }
        double w0 = (yref - y[jj]) * (yref - y[jj + 1]) / ((y[jj - 1] - y[jj]) * (y[jj - 1] - y[jj + 1]));
        double w1 = (yref - y[jj - 1]) * (yref - y[jj + 1]) / ((y[jj] - y[jj - 1]) * (y[jj] - y[jj + 1]));
        double w2 = (yref - y[jj - 1]) * (yref - y[jj]) / ((y[jj + 1] - y[jj - 1]) * (y[jj + 1] - y[jj]));
        for (int i = 1; i <= n1; i++) F3(*ui, i, 1, j) = w0 * F3(*u, i, 1, jj - 1) + w1 * F3(*u, i, 1, jj) + w2 * F3(*u, i, 1, jj + 1);
    }
    for (int e = 0; e < 2; e++) {
        int j = e == 0 ? 1 : n3;
        double yref = yi[j];
        jj = e == 0 ? 2 : ny - 1;
        for (int j2 = 3; j2 <= ny; j2++) if (y[j2] > yref) { jj = j2 - 1; break; }
        double w0 = (yref - y[jj]) * (yref - y[jj + 1]) / ((y[jj - 1] - y[jj]) * (y[jj - 1] - y[jj + 1]));
        double w1 = (yref - y[jj - 1]) * (yref - y[jj + 1]) / ((y[jj] - y[jj - 1]) * (y[jj] - y[jj + 1]));
        double w2 = (yref - y[jj - 1]) * (yref - y[jj]) / ((y[jj + 1] - y[jj - 1]) * (y[jj + 1] - y[jj]));
        for (int i = 1; i <= n1; i++) F3(*ui, i, 1, j) = w0 * F3(*u, i, 1, jj - 1) + w1 * F3(*u, i, 1, jj) + w2 * F3(*u, i, 1, jj + 1);
    }
}

/* interpolate_x_2nd (interpolation.f90:114-179) for u(1:ny,1,1:n3) -> ui(1:n1,1,1:n3) */
static void interp_x_2nd(const double *y, int ny, const fa *u, const double *yi, int n1, fa *ui) {
    int n3 = (int)u->n[2];
    int jj = 2;
    for (int j = 2; j <= n1 - 1; j++) {
        double yref = yi[j];
        for (int j2 = 3; j2 <= ny; j2++) if (y[j2] >= yref) { jj = j2 - 1; break; }
        double w0 = (yref - y[jj]) * (yref - y[jj + 1]) / ((y[jj - 1] - y[jj]) * (y[jj - 1] - y[jj + 1]));
        double w1 = (yref - y[jj - 1]) * (yref - y[jj + 1]) / ((y[jj] - y[jj - 1]) * (y[jj] - y[jj + 1]));
        double w2 = (yref - y[jj - 1]) * (yref - y[jj]) / ((y[jj + 1] - y[jj - 1]) * (y[jj + 1] - y[jj]));
        for (int k = 1; k <= n3; k++) F3(*ui, j, 1, k) = w0 * F3(*u, jj - 1, 1, k) + w1 * F3(*u, jj, 1, k) + w2 * F3(*u, jj + 1, 1, k);
    }
    for (int e = 0; e < 2; e++) {
        int j = e == 0 ? 1 : n1;
        double yref = yi[j];
        jj = e == 0 ? 2 : ny - 1;
        for (int j2 = 3; j2 <= ny; j2++) if (y[j2] >= yref) { jj = j2 - 1; break; }
        if (jj == 0) jj = ny;
        double w0 = (yref - y[jj]) * (yref - y[jj + 1]) / ((y[jj - 1] - y[jj]) * (y[jj - 1] - y[jj + 1]));
        double w1 = (yref - y[jj - 1]) * (yref - y[jj + 1]) / ((y[jj] - y[jj - 1]) * (y[jj] - y[jj + 1]));
        double w2 = (yref - y[jj - 1]) * (yref - y[jj]) / ((y[jj + 1] - y[jj - 1]) * (y[jj + 1] - y[jj]));
        for (int k = 1; k <= n3; k++) F3(*ui, j, 1, k) = w0 * F3(*u, jj - 1, 1, k) + w1 * F3(*u, jj, 1, k) + w2 * F3(*u, jj + 1, 1, k);
    }
}

static void compute_pseudo_pressure_bc_for_robin_bc(cfo *o) {
    /* wallmodel.f90:1342-1378 */
    double *y = o->y, *yg = o->yg;
    int nyg = o->nyg, ny = o->ny, j = 2;
    double a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j]);
    double b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]));
    double c = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1]);
    double Delta_r = (yg[2] - yg[1]) / (yg[3] - yg[2]);
    double alphad = F3(o->alpha_y, 2, 1, 2);
    double beta = alphad / (alphad + y[2] - y[1]);
    double p_bc2 = 1.0 + beta * Delta_r, p_bc3 = -beta * Delta_r;
    F3(o->Dyy, 2, 2, 1) = b + c * p_bc2;
    F3(o->Dyy, 2, 3, 1) = a + c * p_bc3;
    j = nyg - 1;
    a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j]);
    b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]));
    c = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1]);
    alphad = -F3(o->alpha_y, 2, 2, 2);
    Delta_r = (yg[nyg] - yg[nyg - 1]) / (yg[nyg - 1] - yg[nyg - 2]);
    beta = alphad / (alphad - (y[ny] - y[ny - 1]));
    double p_bcn = 1.0 + beta * Delta_r, p_bcn1 = -beta * Delta_r;
    F3(o->Dyy, nyg - 1, nyg - 1, 1) = b + a * p_bcn;
    F3(o->Dyy, nyg - 1, nyg - 2, 1) = c + a * p_bcn1;
}

static void compute_equilibrium_wall_model(cfo *o) {
    /* wallmodel.f90:591-685 */
    int nx = o->nx, nxg = o->nxg, nyg = o->nyg, nz = o->nz, nzg = o->nzg, jref = o->p.jref_eqwm;
    int ncv = o->p.eqwm_ncv > 0 ? o->p.eqwm_ncv : 100;
    double stretch = o->p.eqwm_stretch > 0 ? o->p.eqwm_stretch : 1.10;
    fa *U = &o->U, *W = &o->W, *nt = &o->nu_t;
    for (int k = 1; k <= nz; k++) for (int i = 1; i <= nxg; i++) F3(o->temp_3, i, 1, k) = F3(*W, i, jref, k);
    interp_z_2nd(o->z, nz, &o->temp_3, o->zg, nzg, &o->temp_1);
    interp_x_2nd(o->xg, nxg, &o->temp_1, o->x, nx, &o->temp_2);
    for (int k = 1; k <= nz; k++) for (int i = 1; i <= nxg; i++) F3(o->temp_3, i, 1, k) = F3(*W, i, nyg - jref + 1, k);
    interp_z_2nd(o->z, nz, &o->temp_3, o->zg, nzg, &o->temp_1);
    interp_x_2nd(o->xg, nxg, &o->temp_1, o->x, nx, &o->temp_4);
    int n_nan = 0, n_iter = 0;
    double h = o->yg[jref];
    for (int i = 1; i <= nx; i++)
        for (int k = 1; k <= nzg; k++) {
            for (int wall = 1; wall <= 2; wall++) {
                int jj = wall == 1 ? jref : nyg - jref + 1;
                double wv = wall == 1 ? F3(o->temp_2, i, 1, k) : F3(o->temp_4, i, 1, k);
                double Uv = F3(*U, i, jj, k);
                double u_les = sqrt(Uv * Uv + wv * wv);
                int iter;
                double tau = solve_u_eqwm(u_les, o->nu, 1.0, h, ncv, stretch, &iter, F3(o->tau_eqwm_initial, i, wall, k));
                if (isnan(tau)) { n_nan++; tau = o->tau_mean_eqwm; }
                if (iter == 100) { tau = o->tau_mean_eqwm; n_iter++; }
                F3(o->tau_eqwm_initial, i, wall, k) = tau;
                double tx = tau * Uv / u_les, tz = tau * wv / u_les;
                double nu_t_ik;
                if (wall == 1)
                    nu_t_ik = 0.5 * (0.5 * (F3(*nt, i, 1, k) + F3(*nt, i + 1, 1, k)) + 0.5 * (F3(*nt, i, 2, k) + F3(*nt, i + 1, 2, k)));
                else
                    nu_t_ik = 0.5 * (0.5 * (F3(*nt, i, nyg, k) + F3(*nt, i + 1, nyg, k)) + 0.5 * (F3(*nt, i, nyg - 1, k) + F3(*nt, i + 1, nyg - 1, k)));
                F3(o->alpha_x, i, wall, k) = tx / (o->nu + nu_t_ik);
                F3(o->alpha_z_temp, i, wall, k) = tz / (o->nu + nu_t_ik);
            }
        }
    for (int i = 1; i <= nxg - 2; i++)
        for (int k = 1; k <= nz - 1; k++)
            for (int w = 1; w <= 2; w++)
                F3(o->alpha_z, i, w, k) = 0.25 * (F3(o->alpha_z_temp, i, w, k) + F3(o->alpha_z_temp, i + 1, w, k) +
                                                  F3(o->alpha_z_temp, i, w, k + 1) + F3(o->alpha_z_temp, i + 1, w, k + 1));
    for (int k = 1; k <= nz; k++)
        for (int w = 1; w <= 2; w++) {
            F3(o->alpha_z, nxg, w, k) = F3(o->alpha_z, 3, w, k);
            F3(o->alpha_z, nxg - 1, w, k) = F3(o->alpha_z, 2, w, k);
        }
    for (int i = 1; i <= nxg; i++)
        for (int w = 1; w <= 2; w++) F3(o->alpha_z, i, w, nz) = F3(o->alpha_z, i, w, 2);
    o->n_nan_eqwm = n_nan;
    o->n_iter_eqwm = n_iter;
}

void cfo_compute_wall_model(cfo *o) {
    /* wallmodel.f90:24-82 (iwall_model 0 and 3) */
    if (o->p.iwall_model == 3) compute_equilibrium_wall_model(o);
    if (o->p.iwall_model > 0) compute_pseudo_pressure_bc_for_robin_bc(o);
}

/* ------------------------------------------------------------------------ */
/* Projection, projection.f90                                                */
/* ------------------------------------------------------------------------ */
void cfo_compute_pseudo_pressure_rhs(cfo *o) {
    /* projection.f90:40-55 */
    int nxg = o->nxg, nyg = o->nyg, nzg = o->nzg;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                F3(o->rhs_p, i, j, k) = (F3(o->U, i, j, k) - F3(o->U, i - 1, j, k)) / (o->x[i] - o->x[i - 1]) +
                                        (F3(o->V, i, j, k) - F3(o->V, i, j - 1, k)) / (o->y[j] - o->y[j - 1]) +
                                        (F3(o->W, i, j, k) - F3(o->W, i, j, k - 1)) / (o->z[k] - o->z[k - 1]);
}

void cfo_solve_poisson_equation(cfo *o) {
    /* projection.f90:74-139 */
    int nxp = o->nxp, nzp = o->nzp, nyg = o->nyg, nym = o->nym, nxg = o->nxg, nzg = o->nzg;
    double complex *hat = o->rhs_p_hat; /* (kx, j, kz) with kx fastest */
    for (int j = 2; j <= nyg - 1; j++) {
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) o->plane[(size_t)k * nxp + i] = F3(o->rhs_p, i + 2, j, k + 2);
        fft2d(o->plane, nxp, nzp, o->twx_f, o->twz_f);
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) hat[(size_t)i + (size_t)nxp * ((j - 2) + (size_t)nym * k)] = o->plane[(size_t)k * nxp + i];
    }
#pragma omp parallel
    {
        double complex *D = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
        double complex *DL = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
        double complex *DU = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
        double complex *b = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
#pragma omp for schedule(static)
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) {
                for (int j = 2; j <= nyg - 1; j++) D[j - 2] = F3(o->Dyy, j, j, 1) + o->kxx[i] + o->kzz[k];
                for (int j = 2; j <= nyg - 2; j++) DL[j - 2] = F3(o->Dyy, j + 1, j, 1);
                for (int j = 2; j <= nyg - 2; j++) DU[j - 2] = F3(o->Dyy, j, j + 1, 1);
                if (i == 0 && k == 0) D[0] = 3.0 / 2.0 * D[0];
                for (int j = 0; j < nym; j++) b[j] = hat[(size_t)i + (size_t)nxp * (j + (size_t)nym * k)];
                zgtsv_c(nym, DL, D, DU, b);
                for (int j = 0; j < nym; j++) hat[(size_t)i + (size_t)nxp * (j + (size_t)nym * k)] = b[j];
            }
        free(D); free(DL); free(DU); free(b);
    }
    double norm = (double)((long)nxp * nzp);
    for (int j = 2; j <= nyg - 1; j++) {
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) o->plane[(size_t)k * nxp + i] = hat[(size_t)i + (size_t)nxp * ((j - 2) + (size_t)nym * k)];
        fft2d(o->plane, nxp, nzp, o->twx_b, o->twz_b);
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) F3(o->rhs_p, i + 2, j, k + 2) = creal(o->plane[(size_t)k * nxp + i] / norm);
    }
    /* apply_periodic_xz_pressure, projection.f90:144-162 */
    for (int k = 2; k <= nzg; k++)
        for (int j = 2; j <= nyg - 1; j++) F3(o->rhs_p, nxg - 1, j, k) = F3(o->rhs_p, 2, j, k);
    for (int j = 2; j <= nyg - 1; j++)
        for (int i = 2; i <= nxg - 1; i++) F3(o->rhs_p, i, j, nzp + 2) = F3(o->rhs_p, i, j, 2);
    /* projection.f90:129-137 */
    if (o->rk_step == 1) {
        double f = o->dt * o->rk_coef[1][1];
        for (int k = 2; k <= nzg - 1; k++)
            for (int j = 2; j <= nyg - 1; j++)
                for (int i = 2; i <= nxg - 1; i++) F3(o->P, i, j, k) = F3(o->rhs_p, i, j, k) / f;
        int ny_ = nyg;
        for (int k = 1; k <= nzg; k++) for (int j = 1; j <= ny_; j++) { F3(o->P, 1, j, k) = F3(o->P, 2, j, k); F3(o->P, nxg, j, k) = F3(o->P, nxg - 1, j, k); }
        for (int k = 1; k <= nzg; k++) for (int i = 1; i <= nxg; i++) { F3(o->P, i, 1, k) = F3(o->P, i, 2, k); F3(o->P, i, nyg, k) = F3(o->P, i, nyg - 1, k); }
        for (int j = 1; j <= nyg; j++) for (int i = 1; i <= nxg; i++) { F3(o->P, i, j, 1) = F3(o->P, i, j, 2); F3(o->P, i, j, nzg) = F3(o->P, i, j, nzg - 1); }
    }
}

void cfo_project_velocity(cfo *o) {
    /* projection.f90:203-225 */
    int nx = o->nx, nxg = o->nxg, ny = o->ny, nyg = o->nyg, nz = o->nz, nzg = o->nzg;
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nx - 1; i++)
                F3(o->U, i, j, k) = F3(o->U, i, j, k) - (F3(o->rhs_p, i + 1, j, k) - F3(o->rhs_p, i, j, k)) / (o->xg[i + 1] - o->xg[i]);
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= ny - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                F3(o->V, i, j, k) = F3(o->V, i, j, k) - (F3(o->rhs_p, i, j + 1, k) - F3(o->rhs_p, i, j, k)) / (o->yg[j + 1] - o->yg[j]);
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= nz - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                F3(o->W, i, j, k) = F3(o->W, i, j, k) - (F3(o->rhs_p, i, j, k + 1) - F3(o->rhs_p, i, j, k)) / (o->zg[k + 1] - o->zg[k]);
}

void cfo_compute_projection_step(cfo *o) {
    /* projection.f90:20-28 */
    cfo_compute_pseudo_pressure_rhs(o);
    cfo_solve_poisson_equation(o);
    cfo_project_velocity(o);
}

/* ------------------------------------------------------------------------ */
/* Actual pressure, pressure.f90                                             */
/* ------------------------------------------------------------------------ */
/* bc_1, bc_2 = d/dy(nu dV/dy) at the walls on (2:nxg-1, 2:nzg-1), one-sided
 * 2nd-order derivatives in the index coordinate with metric factors;
 * pressure.f90:270-341. */
static void pressure_bc(cfo *o, fa *bc1, fa *bc2) {
    const double *y = o->y, *yg = o->yg;
    int nxg = o->nxg, nzg = o->nzg, ny = o->ny, nyg = o->nyg;
    double dzeta = 1.0;
    double g = (-3.0 * y[1] + 4.0 * y[2] - y[3]) / (2.0 * dzeta);
    double g2 = (2.0 * y[1] - 5.0 * y[2] + 4.0 * y[3] - 1.0 * y[4]) / pow(dzeta, 2.0);
    double a1 = F3(o->avg_nu_t, 1, 1, 1), a2 = F3(o->avg_nu_t, 1, 2, 1);
    for (int k = 2; k <= nzg - 1; k++)
        for (int i = 2; i <= nxg - 1; i++) {
            double nui = o->nu + 0.5 * (a1 + a2);
            double dnu = (a2 - a1) / (yg[2] - yg[1]);
            double dV = (-3.0 * F3(o->V, i, 1, k) + 4.0 * F3(o->V, i, 2, k) - F3(o->V, i, 3, k)) / (2.0 * dzeta) * 1.0 / g;
            double ddV = (2.0 * F3(o->V, i, 1, k) - 5.0 * F3(o->V, i, 2, k) + 4.0 * F3(o->V, i, 3, k) - 1.0 * F3(o->V, i, 4, k)) /
                         pow(dzeta, 2.0);
            ddV = (ddV - dV * g2) / pow(g, 2.0);
            F3(*bc1, i, k, 1) = dnu * dV + nui * ddV;
        }
    g = (3.0 * y[ny] - 4.0 * y[ny - 1] + y[ny - 2]) / (2.0 * dzeta);
    g2 = (2.0 * y[ny] - 5.0 * y[ny - 1] + 4.0 * y[ny - 2] - 1.0 * y[ny - 3]) / pow(dzeta, 2.0);
    double b1 = F3(o->avg_nu_t, 1, nyg, 1), b2 = F3(o->avg_nu_t, 1, nyg - 1, 1);
    for (int k = 2; k <= nzg - 1; k++)
        for (int i = 2; i <= nxg - 1; i++) {
            double nui = o->nu + 0.5 * (b1 + b2);
            double dnu = (b1 - b2) / (yg[nyg] - yg[nyg - 1]);
            double dV = (3.0 * F3(o->V, i, ny, k) - 4.0 * F3(o->V, i, ny - 1, k) + F3(o->V, i, ny - 2, k)) / (2.0 * dzeta) * 1.0 / g;
            double ddV = (2.0 * F3(o->V, i, ny, k) - 5.0 * F3(o->V, i, ny - 1, k) + 4.0 * F3(o->V, i, ny - 2, k) -
                          1.0 * F3(o->V, i, ny - 3, k)) / pow(dzeta, 2.0);
            ddV = (ddV - dV * g2) / pow(g, 2.0);
            F3(*bc2, i, k, 1) = dnu * dV + nui * ddV;
        }
}

/* 2-D transform of bc(2:nxp+1, 2:nzp+1) into hat (x fastest); pressure.f90:109-115 */
static void bc_hat(cfo *o, fa *bc, double complex *hat) {
    int nxp = o->nxp, nzp = o->nzp;
    for (int k = 0; k < nzp; k++)
        for (int i = 0; i < nxp; i++) hat[(size_t)k * nxp + i] = F3(*bc, i + 2, k + 2, 1);
    fft2d(hat, nxp, nzp, o->twx_f, o->twz_f);
}

void cfo_compute_pressure(cfo *o) {
    /* pressure.f90:21-29 */
    int nx = o->nx, ny = o->ny, nz = o->nz, nxg = o->nxg, nyg = o->nyg, nzg = o->nzg;
    int nxp = o->nxp, nzp = o->nzp, nym = o->nym;
    fa bc1 = fa_new3(2, nxg - 1, 2, nzg - 1, 1, 1), bc2 = fa_new3(2, nxg - 1, 2, nzg - 1, 1, 1);
    pressure_bc(o, &bc1, &bc2);

    /* compute_pressure_rhs, pressure.f90:42-70.  The right-hand sides go to
     * rhs_uf/vf/wf (full extents); the RK slot 1 arrays are borrowed for the
     * calls and left as they were. */
    fa ru = fa_new3(1, nx, 1, nyg, 1, nzg), rv = fa_new3(1, nxg, 1, ny, 1, nzg), rw = fa_new3(1, nxg, 1, nyg, 1, nz);
    fa su = o->Fu[1], sv = o->Fv[1], sw = o->Fw[1];
    o->Fu[1] = fa_new3(2, nx - 1, 2, nyg - 1, 2, nzg - 1);
    o->Fv[1] = fa_new3(2, nxg - 1, 2, ny - 1, 2, nzg - 1);
    o->Fw[1] = fa_new3(2, nxg - 1, 2, nyg - 1, 2, nz - 1);
    cfo_compute_rhs_u(o, 1);
    cfo_compute_rhs_v(o, 1);
    cfo_compute_rhs_w(o, 1);
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nx - 1; i++) F3(ru, i, j, k) = F3(o->Fu[1], i, j, k);
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= ny - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) F3(rv, i, j, k) = F3(o->Fv[1], i, j, k);
    for (int k = 2; k <= nz - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++) F3(rw, i, j, k) = F3(o->Fw[1], i, j, k);
    fa_free(&o->Fu[1]); fa_free(&o->Fv[1]); fa_free(&o->Fw[1]);
    o->Fu[1] = su; o->Fv[1] = sv; o->Fw[1] = sw;
    periodic_x(&ru, 1, nx, nxg, 1);
    for (int k = 2; k <= nzg - 1; k++)
        for (int i = 2; i <= nxg - 1; i++) {
            F3(rv, i, 1, k) = F3(bc1, i, k, 1);   /* compute_rhs_v_boundary, pressure.f90:237-247 */
            F3(rv, i, ny, k) = F3(bc2, i, k, 1);
        }
    periodic_z(&rw, 3, nz, nzg, 1);
    for (size_t q = 0; q < fa_size(&o->rhs_p); q++) o->rhs_p.p[q] = 0.0;
    for (int k = 2; k <= nzg - 1; k++)
        for (int j = 2; j <= nyg - 1; j++)
            for (int i = 2; i <= nxg - 1; i++)
                F3(o->rhs_p, i, j, k) = (F3(ru, i, j, k) - F3(ru, i - 1, j, k)) / (o->x[i] - o->x[i - 1]) +
                                        (F3(rv, i, j, k) - F3(rv, i, j - 1, k)) / (o->y[j] - o->y[j - 1]) +
                                        (F3(rw, i, j, k) - F3(rw, i, j, k - 1)) / (o->z[k] - o->z[k - 1]);
    fa_free(&ru); fa_free(&rv); fa_free(&rw);

    /* solve_poisson_equation_for_pressure, pressure.f90:94-172 */
    double complex *hat = o->rhs_p_hat;
    for (int j = 2; j <= nyg - 1; j++) {
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) o->plane[(size_t)k * nxp + i] = F3(o->rhs_p, i + 2, j, k + 2);
        fft2d(o->plane, nxp, nzp, o->twx_f, o->twz_f);
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) hat[(size_t)i + (size_t)nxp * ((j - 2) + (size_t)nym * k)] = o->plane[(size_t)k * nxp + i];
    }
    double complex *b1h = (double complex *)malloc(sizeof(double complex) * (size_t)nxp * nzp);
    double complex *b2h = (double complex *)malloc(sizeof(double complex) * (size_t)nxp * nzp);
    bc_hat(o, &bc1, b1h);
    bc_hat(o, &bc2, b2h);
    const double e1 = o->coef_bc_1 * (o->yg[2] - o->yg[1]), e2 = o->coef_bc_2 * (o->yg[nyg] - o->yg[nyg - 1]);
#pragma omp parallel
    {
        double complex *D = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
        double complex *DL = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
        double complex *DU = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
        double complex *b = (double complex *)malloc(sizeof(double complex) * (size_t)nym);
#pragma omp for schedule(static)
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) {
                for (int j = 2; j <= nyg - 1; j++) D[j - 2] = F3(o->Dyy, j, j, 1) + o->kxx[i] + o->kzz[k];
                for (int j = 2; j <= nyg - 2; j++) DL[j - 2] = F3(o->Dyy, j + 1, j, 1);
                for (int j = 2; j <= nyg - 2; j++) DU[j - 2] = F3(o->Dyy, j, j + 1, 1);
                if (i == 0 && k == 0) D[0] = 3.0 / 2.0 * D[0];
                for (int j = 0; j < nym; j++) b[j] = hat[(size_t)i + (size_t)nxp * (j + (size_t)nym * k)];
                b[0] = b[0] + e1 * b1h[(size_t)k * nxp + i];
                b[nym - 1] = b[nym - 1] - e2 * b2h[(size_t)k * nxp + i];
                zgtsv_c(nym, DL, D, DU, b);
                for (int j = 0; j < nym; j++) hat[(size_t)i + (size_t)nxp * (j + (size_t)nym * k)] = b[j];
            }
        free(D); free(DL); free(DU); free(b);
    }
    free(b1h); free(b2h);
    double norm = (double)((long)nxp * nzp);
    for (int j = 2; j <= nyg - 1; j++) {
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) o->plane[(size_t)k * nxp + i] = hat[(size_t)i + (size_t)nxp * ((j - 2) + (size_t)nym * k)];
        fft2d(o->plane, nxp, nzp, o->twx_b, o->twz_b);
        for (int k = 0; k < nzp; k++)
            for (int i = 0; i < nxp; i++) F3(o->P, i + 2, j, k + 2) = creal(o->plane[(size_t)k * nxp + i] / norm);
    }
    /* pressure.f90:158-159.  The reference assigns the (nxg-2, nzg-2) array
     * bc_1 to the (nxg, nzg) section P(:,1,:); the restatement applies it on
     * the conforming part i = 2..nxg-1, k = 2..nzg-1 and leaves the x and z
     * ghost columns of rows 1 and nyg as they were. */
    for (int k = 2; k <= nzg - 1; k++)
        for (int i = 2; i <= nxg - 1; i++) {
            F3(o->P, i, 1, k) = F3(o->P, i, 2, k) - (o->yg[2] - o->yg[1]) * F3(bc1, i, k, 1);
            F3(o->P, i, nyg, k) = F3(o->P, i, nyg - 1, k) + (o->yg[nyg] - o->yg[nyg - 1]) * F3(bc2, i, k, 1);
        }
    /* apply_periodic_xz_pressure, pressure.f90:177-195 (one slab); the
     * interior-plane exchange of pressure.f90:200-225 has nothing to do */
    for (int k = 1; k <= nzg; k++)
        for (int j = 1; j <= nyg; j++) F3(o->P, nxg - 1, j, k) = F3(o->P, 2, j, k);
    for (int j = 1; j <= nyg; j++)
        for (int i = 2; i <= nxg - 1; i++) F3(o->P, i, j, nzp + 2) = F3(o->P, i, j, 2);
    fa_free(&bc1); fa_free(&bc2);
}

double cfo_check_divergence(cfo *o, double *maxabs) {
    /* projection.f90:234-256 (signed maximum, plus max |div| for the gate) */
    double div = 0.0, adiv = 0.0;
    for (int k = 2; k <= o->nzg - 1; k++)
        for (int j = 2; j <= o->nyg - 1; j++)
            for (int i = 2; i <= o->nxg - 1; i++) {
                double d = (F3(o->U, i, j, k) - F3(o->U, i - 1, j, k)) / (o->x[i] - o->x[i - 1]) +
                           (F3(o->V, i, j, k) - F3(o->V, i, j - 1, k)) / (o->y[j] - o->y[j - 1]) +
                           (F3(o->W, i, j, k) - F3(o->W, i, j, k - 1)) / (o->z[k] - o->z[k - 1]);
                div = d > div ? d : div;
                adiv = fabs(d) > adiv ? fabs(d) : adiv;
            }
    if (maxabs) *maxabs = adiv;
    return div;
}

/* ------------------------------------------------------------------------ */
/* compute_time_step_RK3, time_integration.f90:89-173                        */
/* ------------------------------------------------------------------------ */
void cfo_time_step_rk3(cfo *o) {
    double to = o->t;
    memcpy(o->Uo.p, o->U.p, fa_size(&o->U) * sizeof(double));
    memcpy(o->Vo.p, o->V.p, fa_size(&o->V) * sizeof(double));
    memcpy(o->Wo.p, o->W.p, fa_size(&o->W) * sizeof(double));
    for (int s = 1; s <= 3; s++) {
        o->rk_step = s;
        cfo_compute_eddy_viscosity(o);
        if (s == 1) {
            cfo_compute_wall_model(o);
            cfo_compute_eddy_viscosity(o);
        }
        cfo_compute_rhs_u(o, s);
        cfo_compute_rhs_v(o, s);
        cfo_compute_rhs_w(o, s);
        cfo_rk_update(o, s);
        o->t = to + o->rk_t[s] * o->dt;
        cfo_apply_boundary_conditions(o);
        cfo_compute_projection_step(o);
        cfo_apply_boundary_conditions(o);
    }
    if (o->p.x_mass_cte == 1 || o->p.x_mass_cte == 2) {
        double dPdx = (o->p.x_mass_cte == 1) ? cfo_compute_dPx_for_constant_mass_flow(o) : compute_dPx_for_constant_Ucenterline(o);
        for (int k = 2; k <= o->nzg - 1; k++)
            for (int j = 2; j <= o->nyg - 1; j++)
                for (int i = 2; i <= o->nx - 1; i++) F3(o->U, i, j, k) = F3(o->U, i, j, k) + dPdx;
        o->dPdx = dPdx / o->dt;
        cfo_apply_boundary_conditions(o);
    }
    if (o->p.y_mass_cte == 1) {
        double dPdy = compute_dPy_for_constant_mass_flow(o);
        for (int k = 2; k <= o->nzg - 1; k++)
            for (int j = 2; j <= o->ny - 1; j++)
                for (int i = 2; i <= o->nxg - 1; i++) F3(o->V, i, j, k) = F3(o->V, i, j, k) + dPdy;
        o->dPdy = dPdy / o->dt;
        cfo_apply_boundary_conditions(o);
    }
}

/* ------------------------------------------------------------------------ */
/* output_monitor reductions, monitor.f90:28-52, 74-81: out[9] = mean U, V, */
/* W, max U, V, W, mean nu_t, max nu_t, max divergence.  Fortran Sum and     */
/* Maxval over column-major sections.                                        */
/* ------------------------------------------------------------------------ */
static void sum_max(fa *F, int i1, int j1, int k1, double *sum, double *mx) {
    double s = 0.0, m = -INFINITY;
    for (int k = 2; k <= k1; k++)
        for (int j = 2; j <= j1; j++)
            for (int i = 2; i <= i1; i++) {
                double v = F3(*F, i, j, k);
                s += v;
                if (v > m) m = v;
            }
    *sum = s;
    *mx = m;
}

void cfo_output_monitor(cfo *o, double *out) {
    int nx = o->nx, ny = o->ny, nz = o->nz, nxg = o->nxg, nyg = o->nyg, nzg = o->nzg;
    double su, sv, sw, sn, mu, mv, mw, mn;
    sum_max(&o->U, nx - 1, nyg - 1, nzg - 1, &su, &mu);
    sum_max(&o->V, nxg - 1, ny - 1, nzg - 1, &sv, &mv);
    sum_max(&o->W, nxg - 1, nyg - 1, nz - 1, &sw, &mw);
    sum_max(&o->nu_t, nxg - 1, nyg - 1, nzg - 1, &sn, &mn);
    double cells = (double)(nx - 1) * (double)(ny - 1) * (double)(nz - 1);
    out[0] = su / cells;
    out[1] = sv / cells;
    out[2] = sw / cells;
    out[3] = mu;
    out[4] = mv;
    out[5] = mw;
    out[6] = sn / ((double)nxg * (double)nyg * (double)nzg);
    out[7] = mn;
    double mabs;
    out[8] = cfo_check_divergence(o, &mabs);
}

/* ------------------------------------------------------------------------ */
/* compute_statistics, statistics.f90:43-159.                                */
/* out layout: 9 profiles of length ny (Umean, Vmean, Wmean, U2, V2, W2, UV,  */
/* Pmean, P2mean) then utau, Retau, Qflow_x, Qflow_y, dUdy_b, dUdy_t,        */
/* nu_t_avg_b, nu_t_avg_t.                                                   */
/* ------------------------------------------------------------------------ */
void cfo_compute_statistics(cfo *o, double *out) {
    int nx = o->nx, nxg = o->nxg, ny = o->ny, nyg = o->nyg, nz = o->nz, nzg = o->nzg;
    const double *w0 = o->weight_y_0, *w1 = o->weight_y_1;
    double *Um = out, *Vm = out + ny, *Wm = out + 2 * ny, *U2 = out + 3 * ny, *V2 = out + 4 * ny, *W2 = out + 5 * ny;
    double *UV = out + 6 * ny, *Pm = out + 7 * ny, *P2 = out + 8 * ny;
    for (int jj = 1; jj <= ny; jj++) {
        double su = 0, su2 = 0, sw = 0, sw2 = 0, sv = 0, sv2 = 0, suv = 0;
        for (int k = 1; k <= nzg - 2; k++)
            for (int i = 1; i <= nx - 2; i++) {
                double t1 = w0[jj] * F3(o->U, i, jj, k) + w1[jj] * F3(o->U, i, jj + 1, k);
                su += t1; su2 += pow(t1, 2.0);
            }
        for (int k = 1; k <= nz - 2; k++)
            for (int i = 1; i <= nxg - 2; i++) {
                double t2 = w0[jj] * F3(o->W, i, jj, k) + w1[jj] * F3(o->W, i, jj + 1, k);
                sw += t2; sw2 += pow(t2, 2.0);
            }
        for (int k = 2; k <= nzg - 1; k++)
            for (int i = 2; i <= nxg - 1; i++) {
                double v = F3(o->V, i, jj, k);
                /* term(i-1) = interpolate_x(term_1) at centre i */
                double ta = w0[jj] * F3(o->U, i - 1, jj, k) + w1[jj] * F3(o->U, i - 1, jj + 1, k);
                double tb = w0[jj] * F3(o->U, i, jj, k) + w1[jj] * F3(o->U, i, jj + 1, k);
                sv += v; sv2 += pow(v, 2.0);
                suv += v * (0.5 * (ta + tb));
            }
        Um[jj - 1] = su / (double)((nx - 2) * (nzg - 2));
        Vm[jj - 1] = sv / (double)((nxg - 2) * (nzg - 2));
        Wm[jj - 1] = sw / (double)((nxg - 2) * (nz - 2));
        U2[jj - 1] = su2 / (double)((nx - 2) * (nzg - 2));
        V2[jj - 1] = sv2 / (double)((nxg - 2) * (nzg - 2));
        W2[jj - 1] = sw2 / (double)((nxg - 2) * (nz - 2));
        UV[jj - 1] = suv / (double)((nxg - 2) * (nzg - 2));
        Pm[jj - 1] = UV[jj - 1] / (double)((nxg - 2) * (nzg - 2)); /* statistics.f90:117 */
        P2[jj - 1] = UV[jj - 1] / (double)((nxg - 2) * (nzg - 2));
    }
    double U1 = 0, Ua = 0, Un1 = 0, Un2 = 0;
    for (int k = 2; k <= nzg - 1; k++)
        for (int i = 2; i <= nx - 1; i++) {
            U1 += F3(o->U, i, 1, k); Ua += F3(o->U, i, 2, k);
            Un1 += F3(o->U, i, nyg - 1, k); Un2 += F3(o->U, i, nyg, k);
        }
    double cnt = (double)((nx - 2) * (nzg - 2));
    U1 /= cnt; Ua /= cnt; Un1 /= cnt; Un2 /= cnt;
    double dUdy_b = (Ua - U1) / (o->yg[2] - o->yg[1]);
    double dUdy_t = (Un2 - Un1) / (o->yg[nyg] - o->yg[nyg - 1]);
    double nb = 0, ntp = 0;
    for (int k = 2; k <= nzg - 1; k++)
        for (int i = 2; i <= nxg - 1; i++) {
            nb += F3(o->nu_t, i, 1, k) + F3(o->nu_t, i, 2, k);
            ntp += F3(o->nu_t, i, nyg - 1, k) + F3(o->nu_t, i, nyg, k);
        }
    nb = nb / (double)((nxg - 2) * (nzg - 2)) / 2.0;
    ntp = ntp / (double)((nxg - 2) * (nzg - 2)) / 2.0;
    double UVb = UV[0], UVt = UV[ny - 1];
    double utau = pow((UVt - UVb - (o->nu + ntp) * dUdy_t + (o->nu + nb) * dUdy_b) / o->Ly, 0.5);
    double Retau = utau * (o->y[ny] - o->y[1]) / 2.0 / o->nu;
    double *tail = out + 9 * ny;
    tail[0] = utau; tail[1] = Retau;
    tail[2] = cfo_compute_mean_mass_flow_U(o);
    tail[3] = cfo_compute_mean_mass_flow_V(o);
    tail[4] = dUdy_b; tail[5] = dUdy_t; tail[6] = nb; tail[7] = ntp;
}
