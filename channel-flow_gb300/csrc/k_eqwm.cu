// k_eqwm.cu -- equilibrium wall model (Larsson), wallmodel.f90:591-685 and
// eqwm.f90:20-223, FP64.
//
// W at the matching row is moved to the U location with the 3-point Lagrange
// interpolations of interpolation.f90:114-252; their stencil choice depends
// only on indices, so the host precomputes (jj, w0, w1, w2) per output index
// with the reference's formulas.  One thread solves the ODE of one wall
// point: Picard iteration on tau_w (<= 101 passes, tol 1e-7), each pass a
// tridiagonal solve over the ncv cells.  The solve eliminates from the top
// (the Dirichlet row, x_ncv = |u|) down to the wall row, so x_1 -- the only
// unknown the stress needs (eqwm.f90:198) -- comes out of one register
// recurrence without storing the Thomas coefficients of eqwm.f90:52-88.
#include "cf_internal.cuh"

// temp_1 = interpolate_z_2nd of W(:, jw, :) at both walls: (nxg, 2, nzg)
template <typename T>
__global__ void k_eq_zinterp_t(Fld<T> W, int jref, int nxg, int nyg, int nzg, const int *zst, const double *zw,
                               double *t1) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int k = blockIdx.y + 1;
    int w = blockIdx.z;
    if (i > nxg) return;
    int jw = w == 0 ? jref : nyg - jref + 1;
    int jj = zst[k];
    const double *c = zw + 3 * k;
    t1[(i - 1) + (long)nxg * (w + 2L * (k - 1))] =
        c[0] * (double)W(i, jw, jj - 1) + c[1] * (double)W(i, jw, jj) + c[2] * (double)W(i, jw, jj + 1);
}

struct EqParams {
    int ncv, jref, nx, nxg, nyg, nzg;
    double nu, h_wm, tau_mean;
    int mixed;  // split path: FP32 Picard passes before the FP64 ones
};

// |u| at the matching row of wall point t = (i, wall, k) (wallmodel.f90:
// 597-612): U there and W moved to the U location by interpolate_x_2nd of
// temp_1; returns u_les and, through Uv / wv, the two components.
struct WallPt {
    int i, w, k, jj;
    long toff;
};
__device__ __forceinline__ WallPt wall_point(long t, const EqParams &ep) {
    WallPt p;
    p.i = (int)(t % ep.nx) + 1;
    const long r = t / ep.nx;
    p.w = (int)(r % 2);
    p.k = (int)(r / 2) + 1;
    p.jj = p.w == 0 ? ep.jref : ep.nyg - ep.jref + 1;
    p.toff = (long)(p.i - 1) + (long)ep.nx * (p.w + 2L * (p.k - 1));
    return p;
}
__device__ __forceinline__ double wall_ules(const WallPt &p, const EqParams &ep, const Fld<double> &Ud, const float *Uf32,
                                            int use_f32, int sy, int sz, const double *t1, const int *xst,
                                            const double *xw, double *Uv_out, double *wv_out) {
    const int xj = xst[p.i];
    const double *c = xw + 3 * p.i;
    const double *row = t1 + (long)ep.nxg * (p.w + 2L * (p.k - 1)) - 1;
    const double wv = c[0] * row[xj - 1] + c[1] * row[xj] + c[2] * row[xj + 1];
    const long uoff = (long)(p.i - 1) + (long)sy * (p.jj - 1) + (long)sz * (p.k - 1);
    const double Uv = use_f32 ? (double)Uf32[uoff] : Ud.p[uoff];
    *Uv_out = Uv;
    *wv_out = wv;
    return sqrt(Uv * Uv + wv * wv);
}

// u_les of every wall point (the input of the learned wall stress)
__global__ void k_wm_ules(const Fld<double> Ud, const float *Uf32, int use_f32, int sy, int sz, const double *t1,
                          const int *xst, const double *xw, EqParams ep, double *ules) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)ep.nx * ep.nzg * 2) return;
    const WallPt p = wall_point(t, ep);
    double Uv, wv;
    ules[p.toff] = wall_ules(p, ep, Ud, Uf32, use_f32, sy, sz, t1, xst, xw, &Uv, &wv);
}

// Learned-stress state of the wall model: the network's stress and envelope
// flag per point, the call counter and checking period, the checked eqwm
// stress.  mode 0: eqwm everywhere (the reference).
struct WmState {
    const double *tau_nn;
    const int *inside;
    const int *calls;
    int check_every;
    int mode;
    double *tau_eq;
};

// Largest ncv for which the split path keeps each point's exponentials of
// the last FP64 pass in shared memory (128 threads x (ncv-1) doubles: 45 KB).
constexpr int EQ_EXP_NCV = 45;
// offset (in doubles) of the kept exponentials: past the grid arrays
__host__ __device__ __forceinline__ int eq_exp_off(int ncv) {
    return (2 * ncv + 3) + ((2 * ncv + 4) * (int)sizeof(float) + 7) / 8;
}

// solve_u_eqwm (eqwm.f90:90-223) inline, grid in shared memory:
// yfa[1..ncv+1], idcv[i] = 1/(y_cv(i+1)-y_cv(i)) (i = 1..ncv-1),
// rw = 1/(y_cv(1)-y_fa(1)); grid[1..ncv] = y_cv, grid[ncv+1..2ncv+1] = y_fa.
// With the learned stress (mode 1) the network's value stands for the solve
// at points inside its training envelope; on checked calls the solve runs for
// every point and its result is kept in tau_eq for the error record.
__global__ void k_eq_solve(const Fld<double> Ud, const float *Uf32, int use_f32, int sy, int sz, const double *t1,
                           const int *xst, const double *xw, const double *grid, EqParams ep, const double *nut,
                           int nut_f32, double *tau0, double *alpha_x, double *alpha_zt, int *counters, WmState wm) {
    extern __shared__ double sg[];
    const int ncv = ep.ncv;
    // grid: yfa[1..ncv+1], idcv[1..ncv-1], rw; FP32 copies after them; then
    // (split path, ncv <= EQ_EXP_NCV) this thread's exponentials of the
    // last FP64 pass, Ex[(q - 2) * blockDim.x + threadIdx.x] for q = 2..ncv
    double *yfa = sg, *idcv = sg + ncv + 2;
    float *yfa32 = (float *)(idcv + ncv + 1), *idcv32 = yfa32 + ncv + 2;
    double *Ex = sg + eq_exp_off(ncv) + threadIdx.x;
    const int exs = blockDim.x;
    const bool keep_ex = ep.mixed && ncv <= EQ_EXP_NCV;
    for (int q = threadIdx.x; q < ncv + 2; q += blockDim.x) {
        yfa[q] = q >= 1 && q <= ncv + 1 ? grid[ncv + q] : 0.0;
        yfa32[q] = (float)yfa[q];
    }
    for (int q = threadIdx.x; q < ncv + 1; q += blockDim.x) {
        idcv[q] = (q >= 1 && q <= ncv - 1) ? 1.0 / (grid[q + 1] - grid[q]) : 0.0;
        idcv32[q] = (float)idcv[q];
    }
    __syncthreads();
    const double rw = 1.0 / (grid[1] - grid[ncv + 1]);
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long npts = (long)ep.nx * ep.nzg * 2;
    if (t >= npts) return;
    const WallPt pt = wall_point(t, ep);
    const int i = pt.i, w = pt.w, k = pt.k;
    const int nxg = ep.nxg, nyg = ep.nyg;
    double Uv, wv;
    const double u_les = wall_ules(pt, ep, Ud, Uf32, use_f32, sy, sz, t1, xst, xw, &Uv, &wv);
    const long toff = pt.toff;
    const bool served = wm.mode == 1 && wm.inside[toff] != 0;
    const bool check = wm.mode == 1 && wm.check_every > 0 && (*wm.calls % wm.check_every) == 0;
    double tau = tau0[toff];
    if (!served || check) {
        // solve_u_eqwm(u_les, nu, 1.0, yg(jref), ncv, stretch, tau, iter, tau_in)
        const double kappa = 0.41, Aplus = 17.0, tol = 0.0000001, mu_lam = ep.nu, rho = 1.0;
        const int max_iter = 100;
        double tau_lam = mu_lam * u_les / ep.h_wm;
        int iter = 0;
        bool mixed_ok = false;  // the FP32 passes gave the FP64 ones their start
        if (ep.mixed) {
            // Split path: the same Picard passes in FP32 (at most 50) until
            // the change is below 1e-5 of tau (FP32 resolves about 1e-7), the
            // unconverged ones counted like FP64 passes; the FP64 passes
            // below then start next to the fixed point and reach the
            // reference's criterion after a few passes, instead of all of
            // them in FP64 (each FP64 pass costs dozens of FP32 ones here).
            // A non-finite or non-positive FP32 result starts the FP64
            // passes from the initial tau instead.
            const float mu32 = (float)mu_lam, ul32 = (float)u_les, rw32 = (float)rw;
            const float c0 = (float)(rho * kappa), cdf = (float)(1.0 / (mu_lam / rho) / Aplus);
            float t = (float)tau;
            int it = 0;
            while (it < 50) {
                const float tp = t, ut = sqrtf(t), c1 = c0 * ut, cd = ut * cdf;
                float al = ul32, be = 0.f, yf = yfa32[ncv];
                float D = 1.f - __expf(-(yf * cd));
                float mu_up = mu32 + c1 * yf * (D * D);
                for (int q = ncv - 1; q >= 2; q--) {
                    yf = yfa32[q];
                    D = 1.f - __expf(-(yf * cd));
                    const float mu_q = mu32 + c1 * yf * (D * D);
                    const float sup = mu_up * idcv32[q], sub = mu_q * idcv32[q - 1];
                    const float rm = 1.f / (-(sup + sub) + sup * be);
                    al = -sup * al * rm;
                    be = -sub * rm;
                    mu_up = mu_q;
                }
                const float sup = mu_up * idcv32[1];
                const float x1 = -sup * al / (-(sup + mu32 * rw32) + sup * be);
                t = mu32 * x1 * rw32;
                if (fabsf(t - tp) < 1e-5f * fabsf(t)) break;
                it++;
            }
            if (isfinite(t) && t > 0.f) {
                tau = (double)t;
                iter = it;
                mixed_ok = true;
            }
        }
        // one FP64 Picard pass of solve_u_eqwm (eqwm.f90:121-205): tau from
        // the mixing-length viscosity of the previous tau.  In the split path
        // (keep_ex) a pass whose factor cd differs from the last pass's by
        // |dcd| yfa[ncv] <= 1e-3 takes exp(-(y cd)) as the last pass's value
        // times exp(-(y dcd)), the latter as its degree-4 Taylor polynomial
        // (truncation below 1e-17 relative), instead of evaluating exp; and
        // the elimination runs in continuant form (below), as accurate as the
        // division per cell of the reference's Thomas sweep (both within a
        // few 1e-14 of exact rational elimination on the same coefficients
        // at ncv 30).
        double cd_last = -1.0;  // no exponentials kept yet
        auto pass64 = [&](double tau) -> double {
            double nu_eq = mu_lam / rho;
            double utau = sqrt(tau / rho);
            double c1 = rho * kappa * utau;
            // y utau / nu / A+ of eqwm.f90:134-136 with the per-pass factor
            // formed once (two FP64 divisions less per cell)
            const double cd = utau / nu_eq / Aplus;
            const double dcd = cd - cd_last;
            const double xmax = fabs(dcd) * yfa[ncv];
            const bool upd = keep_ex && cd_last >= 0.0 && xmax <= 1e-3, low = xmax <= 1e-6;
            if (keep_ex) cd_last = cd;
            auto ex = [&](int q, double yf) -> double {
                double e;
                if (upd) {
                    // |x| <= 1e-6: degree 2 (truncation x^3/6 < 2e-19)
                    const double x = -(yf * dcd);
                    const double p = low ? 1.0 + x * (1.0 + 0.5 * x)
                                         : 1.0 + x * (1.0 + x * (0.5 + x * (1.0 / 6.0 + x * (1.0 / 24.0))));
                    e = Ex[(q - 2) * exs] * p;
                } else {
                    e = exp(-(yf * cd));
                }
                if (keep_ex) Ex[(q - 2) * exs] = e;
                return e;
            };
            double yf = yfa[ncv];
            double D = 1.0 - ex(ncv, yf);
            double mu_up = mu_lam + c1 * yf * (D * D);
            if (!ep.mixed) {
                double al = u_les, be = 0.0;
                for (int q = ncv - 1; q >= 2; q--) {
                    yf = yfa[q];
                    D = 1.0 - ex(q, yf);
                    double mu_q = mu_lam + c1 * yf * (D * D);
                    double sup = mu_up * idcv[q];
                    double sub = mu_q * idcv[q - 1];
                    double m = -1.0 * (sup + sub) + sup * be;
                    double rm = 1.0 / m;
                    al = -sup * al * rm;
                    be = -sub * rm;
                    mu_up = mu_q;
                }
                double sup = mu_up * idcv[1];
                double diag = -1.0 * (sup + mu_lam * rw);
                double x1 = -sup * al / (diag + sup * be);
                return mu_lam * (x1 - 0.0) * rw;
            }
            // Split path: the same elimination without a division per cell.
            // With the pivots m_q = Dn_q / Dn_{q+1} (Dn_ncv = 1) the
            // continuants follow Dn_q = -(sup_q + sub_q) Dn_{q+1} -
            // sup_q sub_{q+1} Dn_{q+2}, and A_q = al_q Dn_q = -sup_q A_{q+1};
            // be_2 = -sub_2 Dn_3 / Dn_2, al_2 = A_2 / Dn_2, so the first cell's
            // unknown is one quotient.  sup_q = sub_{q+1} (both mu_{q+1} /
            // (y_cv(q+1) - y_cv(q))).  Dn, A are rescaled by powers of two
            // (exact) every 8 cells to stay in range.
            double Dn1 = 1.0, Dn2 = 0.0, A = u_les, subp = 0.0;
            double sup = mu_up * idcv[ncv - 1];
            for (int q = ncv - 1; q >= 2; q--) {
                yf = yfa[q];
                D = 1.0 - ex(q, yf);
                const double mu_q = mu_lam + c1 * yf * (D * D);
                const double sub = mu_q * idcv[q - 1];
                const double Dn = fma(-(sup + sub), Dn1, -(sup * subp) * Dn2);
                A = -sup * A;
                Dn2 = Dn1;
                Dn1 = Dn;
                subp = sub;
                sup = sub;
                if ((q & 7) == 0) {
                    const int e = ((__double2hiint(Dn1) >> 20) & 0x7ff) - 1023;
                    if (e > 512 || e < -512) {
                        const double sc = __hiloint2double((1023 - e) << 20, 0);  // 2^-e
                        Dn1 *= sc;
                        Dn2 *= sc;
                        A *= sc;
                    }
                }
            }
            // sup = mu_2 / (y_cv(2) - y_cv(1)) of the first cell
            const double diag = -1.0 * (sup + mu_lam * rw);
            const double x1 = -sup * A / (diag * Dn1 - sup * subp * Dn2);
            return mu_lam * x1 * rw;
        };
        bool fin = false;
        if (ep.mixed && mixed_ok) {
            // Split path, from the FP32 iterate: two FP64 passes (checked and
            // counted like the reference's), then Aitken's extrapolation of
            // the linearly converging sequence; the reference passes below
            // take it from there to the reference's criterion.
            const double t0 = tau, t1 = pass64(t0);
            if (fabs((t1 - t0) / tau_lam) < tol) {
                tau = t1;
                fin = true;
            } else {
                iter = iter + 1;
                const double t2 = pass64(t1);
                if (fabs((t2 - t1) / tau_lam) < tol) {
                    tau = t2;
                    fin = true;
                } else {
                    iter = iter + 1;
                    const double d1 = t1 - t0, d2 = t2 - t1, den = d2 - d1;
                    const double ta = den != 0.0 ? t2 - d2 * d2 / den : t2;
                    tau = (isfinite(ta) && ta > 0.0) ? ta : t2;
                }
            }
        }
        while (!fin) {
            double tau_prev = tau;
            tau = pass64(tau);
            int done = 0;
            if (fabs((tau - tau_prev) / tau_lam) < tol) done = 1;
            if (done == 0) iter = iter + 1;
            if (iter > max_iter) done = 1;
            if (done) break;
        }
        // wallmodel.f90:620-640
        if (isnan(tau)) {
            atomicAdd(&counters[0], 1);
            tau = ep.tau_mean;
        }
        if (iter == 100) {
            tau = ep.tau_mean;
            atomicAdd(&counters[1], 1);
        }
        if (check) wm.tau_eq[toff] = tau;
    }
    if (served) tau = wm.tau_nn[toff];
    tau0[toff] = tau;
    double tx = tau * Uv / u_les, tz = tau * wv / u_les;
    int ja = w == 0 ? 1 : nyg, jb = w == 0 ? 2 : nyg - 1;
    long cs = (long)nxg * nyg;
    auto NT = [&](int ii, int j) -> double {
        long o = (long)(ii - 1) + (long)nxg * (j - 1) + cs * (k - 1);
        return nut_f32 ? (double)((const float *)nut)[o] : nut[o];
    };
    double nu_t_ik = 0.5 * (0.5 * (NT(i, ja) + NT(i + 1, ja)) + 0.5 * (NT(i, jb) + NT(i + 1, jb)));
    alpha_x[toff] = tx / (ep.nu + nu_t_ik);
    alpha_zt[toff] = tz / (ep.nu + nu_t_ik);
}

// The error record of checked calls: max and mean |tau_nn/tau_eq - 1| over
// the points the network served, their count and the fallback count; every
// call advances the call counter.  One block.
__global__ void __launch_bounds__(1024) k_wm_audit(long npts, const double *tau_nn, const int *inside,
                                                  const double *tau_eq, int *calls, int check_every, double *log) {
    __shared__ double sm[3][32];
    const bool check = check_every > 0 && (*calls % check_every) == 0;
    if (check) {
        double mx = 0.0, sum = 0.0, cnt = 0.0;
        for (long t = threadIdx.x; t < npts; t += blockDim.x) {
            if (!inside[t]) continue;
            const double e = fabs(tau_nn[t] / tau_eq[t] - 1.0);
            mx = fmax(mx, e);
            sum += e;
            cnt += 1.0;
        }
        for (int o = 16; o > 0; o >>= 1) {
            mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
            sum += __shfl_down_sync(0xffffffffu, sum, o);
            cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        }
        if ((threadIdx.x & 31) == 0) {
            sm[0][threadIdx.x >> 5] = mx;
            sm[1][threadIdx.x >> 5] = sum;
            sm[2][threadIdx.x >> 5] = cnt;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int q = 1; q < (int)(blockDim.x >> 5); q++) {
                mx = fmax(mx, sm[0][q]);
                sum += sm[1][q];
                cnt += sm[2][q];
            }
            log[0] = (double)(*calls + 1);
            log[1] = mx;
            log[2] = cnt > 0 ? sum / cnt : 0.0;
            log[3] = cnt;
            log[4] = (double)npts - cnt;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *calls = *calls + 1;
}

// alpha_z: 4-point average of alpha_z_temp and its copies (wallmodel.f90:656-664)
__global__ void k_eq_alphaz(const double *azt, double *az, int nx, int nxg, int nz, int nzg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int k = blockIdx.y + 1;
    int w = blockIdx.z;
    if (i > nxg) return;
    // value of alpha_z(i,w,k) after the three copy statements
    int ii = i, kk = k;
    if (kk == nz) kk = 2;
    if (ii == nxg) ii = 3;
    else if (ii == nxg - 1) ii = 2;
    auto T = [&](int a, int c) { return azt[(a - 1) + (long)nx * (w + 2L * (c - 1))]; };
    double v = 0.25 * (T(ii, kk) + T(ii + 1, kk) + T(ii, kk + 1) + T(ii + 1, kk + 1));
    az[(i - 1) + (long)nxg * (w + 2L * (k - 1))] = v;
}

template <typename T>
int launch_eqwm(cf_ctx *ctx, int b) {
    if (int rc = launch_nut_wall_rows<T>(ctx)) return rc;  // the rows k_eq_solve reads
    int nx = ctx->nx, nxg = ctx->nxg, nyg = ctx->nyg, nz = ctx->nz, nzg = ctx->nzg;
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    k_eq_zinterp_t<T><<<dim3(cdiv(nxg, 128), nzg, 2), 128, 0, ctx->st>>>(W, ctx->prm.jref_eqwm, nxg, nyg, nzg,
                                                                         ctx->eq_zst, ctx->eq_zw, ctx->wtemp1);
    count_launch(ctx, "k_eq_zinterp_t");
    EqParams ep;
    ep.ncv = ctx->prm.eqwm_ncv;
    ep.jref = ctx->prm.jref_eqwm;
    ep.nx = nx; ep.nxg = nxg; ep.nyg = nyg; ep.nzg = nzg;
    ep.nu = ctx->prm.nu;
    ep.h_wm = ctx->hyg[ep.jref];
    ep.tau_mean = ctx->hs.tau_mean_eqwm;
    ep.mixed = sizeof(T) == 4;
    CF_CUDA(cudaMemsetAsync(ctx->d_red, 0, 2 * sizeof(int), ctx->st));
    long npts = (long)nx * nzg * 2;
    size_t sh = (size_t)eq_exp_off(ep.ncv) * sizeof(double);
    if (ep.mixed && ep.ncv <= EQ_EXP_NCV) sh += (size_t)(ep.ncv - 1) * 128 * sizeof(double);
    Fld<double> Ud = make_fld<double>(ctx->U[b], nx, nyg);
    WmState wm = {};
    if (ctx->wmlp) {
        // the learned stress of every point, then the solve where it does not serve
        k_wm_ules<<<cdiv(npts, 256), 256, 0, ctx->st>>>(Ud, (const float *)ctx->U[b], sizeof(T) == 4, nx, nx * nyg,
                                                        ctx->wtemp1, ctx->eq_xst, ctx->eq_xw, ep, ctx->wm_u);
        count_launch(ctx, "k_wm_ules");
        if (int rc = wall_mlp_infer(ctx, (int)npts, ep.h_wm, ep.nu)) return rc;
        wm.tau_nn = ctx->wm_tau;
        wm.inside = ctx->wm_inside;
        wm.calls = ctx->wm_calls;
        wm.check_every = ctx->wm_check_every;
        wm.mode = 1;
        wm.tau_eq = ctx->wm_tau_eq;
    }
    k_eq_solve<<<cdiv(npts, 128), 128, sh, ctx->st>>>(Ud, (const float *)ctx->U[b], sizeof(T) == 4, nx, nx * nyg,
                                                     ctx->wtemp1, ctx->eq_xst, ctx->eq_xw, ctx->eq_grid, ep,
                                                     (const double *)ctx->nut, sizeof(T) == 4, ctx->tau0, ctx->alpha_x,
                                                     ctx->alpha_zt, (int *)ctx->d_red, wm);
    count_launch(ctx, "k_eq_solve");
    if (ctx->wmlp) {
        k_wm_audit<<<1, 1024, 0, ctx->st>>>(npts, ctx->wm_tau, ctx->wm_inside, ctx->wm_tau_eq, ctx->wm_calls,
                                            ctx->wm_check_every, ctx->wm_log);
        count_launch(ctx, "k_wm_audit");
    }
    k_eq_alphaz<<<dim3(cdiv(nxg, 128), nz, 2), 128, 0, ctx->st>>>(ctx->alpha_zt, ctx->alpha_z, nx, nxg, nz, nzg);
    count_launch(ctx, "k_eq_alphaz");
    CF_CUDA(cudaGetLastError());
    return 0;
}

template int launch_eqwm<double>(cf_ctx *, int);
template int launch_eqwm<float>(cf_ctx *, int);

// The matching-plane velocity |u| of every wall point for state buffer b --
// the input the wall model hands to the eqwm solve (wallmodel.f90:597-621) --
// into ules (device, nx * 2 * nzg values, wall-point order (i, wall, k)).
template <typename T>
int launch_wm_inputs(cf_ctx *ctx, int b, double *ules) {
    int nx = ctx->nx, nxg = ctx->nxg, nyg = ctx->nyg, nzg = ctx->nzg;
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    k_eq_zinterp_t<T><<<dim3(cdiv(nxg, 128), nzg, 2), 128, 0, ctx->st>>>(W, ctx->prm.jref_eqwm, nxg, nyg, nzg,
                                                                         ctx->eq_zst, ctx->eq_zw, ctx->wtemp1);
    EqParams ep = {};
    ep.ncv = ctx->prm.eqwm_ncv;
    ep.jref = ctx->prm.jref_eqwm;
    ep.nx = nx; ep.nxg = nxg; ep.nyg = nyg; ep.nzg = nzg;
    ep.nu = ctx->prm.nu;
    ep.h_wm = ctx->hyg[ep.jref];
    const long npts = (long)nx * nzg * 2;
    Fld<double> Ud = make_fld<double>(ctx->U[b], nx, nyg);
    k_wm_ules<<<cdiv(npts, 256), 256, 0, ctx->st>>>(Ud, (const float *)ctx->U[b], sizeof(T) == 4, nx, nx * nyg,
                                                    ctx->wtemp1, ctx->eq_xst, ctx->eq_xw, ep, ules);
    CF_CUDA(cudaGetLastError());
    return 0;
}

template int launch_wm_inputs<double>(cf_ctx *, int, double *);
template int launch_wm_inputs<float>(cf_ctx *, int, double *);
