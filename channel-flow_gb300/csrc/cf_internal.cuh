// cf_internal.cuh -- shared definitions of the channel RK3-substep library.
//
// Device layout: every field keeps the reference's Fortran extents and order
// (initialization.f90:121-152), 1-based indices, x fastest:
//   U (nx,nyg,nzg)  V (nxg,ny,nzg)  W (nxg,nyg,nz)  P, nu_t (nxg,nyg,nzg)
// with nxg = nx+1 etc.  Ghost layers and the periodic duplicate planes are
// stored, so a kernel reads exactly the values the reference reads.
// Quantities the reference only keeps periodic copies of (the eddy-viscosity
// intermediates, the pseudo-pressure) live in a compact "canonical" layout of
// the nxp x nym x nzp unique cells (i = 2..nx-1, j = 2..nyg-1, k = 2..nz-1),
// read through the periodic wrap  i -> 2 + (i-2) mod nxp.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "channel_gpu.h"

#define CF_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            return cf_fail(ctx, CF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                              \
    } while (0)

// Fortran-layout 3-D field view with 1-based indices.
template <typename T>
struct Fld {
    T *p;
    int sy, sz, off;  // off = 1 + sy + sz
    __host__ __device__ __forceinline__ T &operator()(int i, int j, int k) const {
        return p[i + sy * j + sz * k - off];
    }
    __host__ __device__ __forceinline__ int idx(int i, int j, int k) const { return i + sy * j + sz * k - off; }
};

template <typename T>
__host__ __device__ static inline Fld<T> make_fld(void *p, int n1, int n2) {
    Fld<T> f;
    f.p = (T *)p;
    f.sy = n1;
    f.sz = n1 * n2;
    f.off = 1 + f.sy + f.sz;
    return f;
}

// Grid geometry (device pointers, 1-based: x[1..nx]); T = double or float.
template <typename T>
struct GeoT {
    int nx, ny, nz, nxg, nyg, nzg, nxp, nym, nzp, nxh;
    const T *x, *y, *z, *xg, *yg, *zg, *w0, *w1;
};
typedef GeoT<double> Geo;

// Reciprocal spacings r[e] = 1/(a[e] - a[e-1]) (e >= 2) of the face (x, y, z)
// and centre (xg, yg, zg) coordinates, 1-based like the coordinates.
template <typename T>
struct RcpT {
    const T *dx, *dxg, *dy, *dyg, *dz, *dzg;
};

// Device-resident scalars (module globals of global.f90 touched per step).
struct DevScal {
    double dt, t, dPdx, dPdy, dPdz;
    double Qflow_x_0, Qflow_y_0, Ucenterline_x, tau_mean_eqwm;
    double lmax[3];        // compute_dt maxima (bit patterns ordered as int64)
    double mass_sum;       // mass-flow integral
    double fixed_dt;       // > 0: dt forced (CFL < 0 rule)
    int rk_step, n_nan, n_iter;
    int n_wait;            // plane copies whose bounded wait expired (filter kernel)
    // FP32 copies for the split path (written next to their FP64 values)
    float dtf, dPdxf, dPdzf, corrf;
};

template <typename T> __device__ __forceinline__ T ds_dt(const DevScal *d);
template <> __device__ __forceinline__ double ds_dt<double>(const DevScal *d) { return d->dt; }
template <> __device__ __forceinline__ float ds_dt<float>(const DevScal *d) { return d->dtf; }
template <typename T> __device__ __forceinline__ T ds_dpdx(const DevScal *d);
template <> __device__ __forceinline__ double ds_dpdx<double>(const DevScal *d) { return d->dPdx; }
template <> __device__ __forceinline__ float ds_dpdx<float>(const DevScal *d) { return d->dPdxf; }
template <typename T> __device__ __forceinline__ T ds_dpdz(const DevScal *d);
template <> __device__ __forceinline__ double ds_dpdz<double>(const DevScal *d) { return d->dPdz; }
template <> __device__ __forceinline__ float ds_dpdz<float>(const DevScal *d) { return d->dPdzf; }

// Compensated (float-float) state of the split path: hi + lo holds a value
// to about 2^-48 relative; updates use Knuth's TwoSum so that no FP64
// arithmetic runs per grid point (GB300's FP64 rate is ~1/40 of FP32).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// (hi, lo) += d, renormalised
__device__ __forceinline__ void ff_add(float &hi, float &lo, float d) {
    float s, e;
    two_sum(hi, d, s, e);
    e += lo;
    hi = s + e;
    lo = e - (hi - s);
}
// (hi, lo) += (bh, bl), both float-float
__device__ __forceinline__ void ff_add2(float &hi, float &lo, float bh, float bl) {
    float s, e;
    two_sum(hi, bh, s, e);
    e += lo + bl;
    hi = s + e;
    lo = e - (hi - s);
}

// periodic index for i in [2 - np, 2 np + 1] (compares only)
__host__ __device__ __forceinline__ int wrapn(int i, int np) { return i < 2 ? i + np : (i > np + 1 ? i - np : i); }

__host__ __device__ __forceinline__ int wrapc(int i, int np) {
    // canonical index of a periodic index (faces or centres): 2 + (i-2) mod np
    int r = (i - 2) % np;
    if (r < 0) r += np;
    return 2 + r;
}

static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

// The seam band of the wall-model configurations.  With the equilibrium wall
// model the wall ghost rows of U and W (j = 1, nyg) are not periodic copies at
// the seam columns and planes (their Neumann values use alpha at the ghost's
// own position).  The reference reads those entries themselves in the
// stencils of the canonical centres next to a seam and the canonical twin's
// values where it fills ghost points (subgrid.f90:448-458), while this pass
// reads every halo through the periodic wrap.  A centre's L.M, M.M and |S|
// read U, V, W within two cells of it (through its neighbours' quantities and
// the filtered velocities), so the centres that can see a wall ghost entry
// outside the canonical columns and planes -- rows 2, 3, nyg-2, nyg-1 at
// columns 2, 3, nxp, nxp+1 or planes 2, 3, nzp, nzp+1 -- are computed by
// k_dsm_seam with the reference's readings.
__host__ __device__ __forceinline__ bool seam_row(int j, int nyg) { return j <= 3 || j >= nyg - 2; }
__host__ __device__ __forceinline__ bool seam_line(int i, int np) { return i <= 3 || i >= np; }


// compute_Sij at one centre (subgrid.f90:891-949) from arrays at actual
// indices (any accessor with operator()(i, j, k)).  FP64 divides by the
// spacings as the reference does; FP32 (the split path) multiplies by the
// stored reciprocal spacings rc.
template <typename T, typename A>
__device__ __forceinline__ void sij_point_a(const GeoT<T> &g, const RcpT<T> &rc, const A &U, const A &V, const A &W,
                                            int i, int j, int k, T s[6], T &S) {
    const T *x = g.x, *y = g.y, *z = g.z, *xg = g.xg, *yg = g.yg, *zg = g.zg;
    const T h = T(0.5), q = T(0.25);
    auto quo = [&](T a, const T *c, const T *r, int e) -> T {
        if constexpr (sizeof(T) == 8) return a / (c[e] - c[e - 1]);
        else return a * r[e];
    };
    s[0] = quo(U(i, j, k) - U(i - 1, j, k), x, rc.dx, i);
    s[1] = quo(V(i, j, k) - V(i, j - 1, k), y, rc.dy, j);
    s[2] = quo(W(i, j, k) - W(i, j, k - 1), z, rc.dz, k);
    T e4[2][2], e5[2][2], e6[2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
            int ii = i + a, jj = j + b, kk = k + b;
            // edge values at (ii, jj, k), (ii, j, kk), (i, j+a, k+b)
            e4[a][b] = h * (quo(U(ii - 1, jj, k) - U(ii - 1, jj - 1, k), yg, rc.dyg, jj) +
                            quo(V(ii, jj - 1, k) - V(ii - 1, jj - 1, k), xg, rc.dxg, ii));
            e5[a][b] = h * (quo(U(ii - 1, j, kk) - U(ii - 1, j, kk - 1), zg, rc.dzg, kk) +
                            quo(W(ii, j, kk - 1) - W(ii - 1, j, kk - 1), xg, rc.dxg, ii));
            int j6 = j + a, k6 = k + b;
            e6[a][b] = h * (quo(V(i, j6 - 1, k6) - V(i, j6 - 1, k6 - 1), zg, rc.dzg, k6) +
                            quo(W(i, j6, k6 - 1) - W(i, j6 - 1, k6 - 1), yg, rc.dyg, j6));
        }
    s[3] = q * (e4[0][0] + e4[1][0] + e4[0][1] + e4[1][1]);
    s[4] = q * (e5[0][0] + e5[1][0] + e5[0][1] + e5[1][1]);
    s[5] = q * (e6[0][0] + e6[1][0] + e6[0][1] + e6[1][1]);
    T a2 = T(0);
#pragma unroll
    for (int c = 0; c < 6; c++) a2 += (c < 3 ? T(2) : T(4)) * s[c] * s[c];
    S = sqrt(a2);
}
template <typename T>
__device__ __forceinline__ void sij_point(const GeoT<T> &g, const RcpT<T> &rc, const Fld<T> &U, const Fld<T> &V,
                                          const Fld<T> &W, int i, int j, int k, T s[6], T &S) {
    sij_point_a<T, Fld<T>>(g, rc, U, V, W, i, j, k, s, S);
}


struct cf_ctx {
    int dev = 0;
    cf_params prm;
    int nx, ny, nz, nxg, nyg, nzg, nxp, nym, nzp, nxh;
    size_t nU, nV, nW, nC, nCan, nSpec;
    cudaStream_t st = nullptr;
    std::string err;

    // host geometry (1-based vectors)
    std::vector<double> hx, hy, hz, hxg, hyg, hzg, hw0, hw1, hkxx, hkzz;
    std::vector<double> Dd, Dl, Du;  // tridiagonal rows of Dyy (2..nyg-1)
    double dxmin, dymin, dzmin, Lx, Ly, Lz, mass_norm, omega_z;
    double *d_geo = nullptr;
    float *d_geo_f = nullptr;
    double *d_rgeo = nullptr;          // reciprocal spacings (see rgeo_off)
    float *d_rgeo_f = nullptr;
    size_t rgeo_off[6] = {};
    Geo geo;
    GeoT<float> geof;
    double mass_norm_vv = 1.0;

    // state (element type: double for FP64, float for the split path)
    int esz = 8;                       // bytes per state element
    void *U[3] = {}, *V[3] = {}, *W[3] = {};
    void *Ulo[3] = {}, *Vlo[3] = {}, *Wlo[3] = {};  // split path: low words
    int cur = 0, old = 0;              // current state and Uo buffers
    void *nut = nullptr, *P = nullptr;
    void *F[3][3] = {};                // [slot 0..2][comp]
    // eddy viscosity
    void *dsm_q = nullptr;             // 16 canonical arrays
    void *Uf = nullptr, *Vf = nullptr, *Wf = nullptr;
    double *dsm_part = nullptr;        // plane partial sums
    double *avg_nu_t = nullptr;        // (nyg) device
    int dsm_nblk = 0;
    int dsm_kc = 0;                    // z-chunk length of the fused pass
    int dsm_nchunk_fused = 0;          // plane-partial slots per row of the last one-pass launch
    int dsm_nchunk_base = 0;           // of them, the one-pass kernel's (the seam band's follow)
    bool use_fused_dsm = true;
    int dsmb_nkc = 0;                  // z chunks of the multi-pass DSM filter kernel
    // tensor map (a CUtensorMap) of the 15 filter quantities of dsm_q for the
    // filter kernel's tensor-copy gather; state 0 not tried, 1 encoded, -1 not
    // applicable.  dsmb_skip_first: test hook, the first plane copy of every
    // block is left out so that its bounded wait expires.
    alignas(64) unsigned char dsmb_map[128] = {};
    int dsmb_map_state = 0;
    int dsmb_skip_first = 0;
    bool use_rhs3 = true;              // one fused RHS + update launch per substep
    int rhs_nkc = 1;                   // z chunks of the fused RHS
    int amd_nkc = 1;                   // z chunks of the AMD pass
    int seg_base = 0;                  // buffer a step in segments started from
    size_t dsm_part_nch = 0;           // plane-partial slots per row allocated in dsm_part
    int amd_nparts = 0;                // partial sums per row of the last AMD pass
    bool amd_avg_pending = false;      // avg_nu_t not yet formed from them
    // U, V, W hold the ghosts apply_boundary_conditions gives them: periodic
    // copies in x and z (with the wall model: except the wall ghost rows of U
    // and W at the seams) and the wall rule
    bool state_periodic = false;
    // After the one-pass eddy viscosity, nu_t is held as |S| (canonical) and
    // the plane coefficient <LM>/<MM>: the fused RHS forms nu_t on the fly and
    // the nut buffer is filled only when another reader needs it.
    bool nut_lazy = false;
    // pressure
    void *phi = nullptr;               // canonical real
    void *spec = nullptr;              // complex spectrum [j][kz][kx]: mode m = kz*nxh + kx contiguous per row
    double *d_tri = nullptr;           // Dd, Dl, Du (nym each), kxx (nxp), kzz (nzp)
    double *tri_fac = nullptr;         // zgtsv factors [row][mode]: m, 1/d, du, dl
    unsigned char *tri_piv = nullptr;  // zgtsv pivot flags [row][mode]
    // split path: FP32 LU factors of the modes whose elimination never pivots
    float *tri_l32 = nullptr;          // multipliers [row][mode]
    float *tri_ru32 = nullptr;         // 1/d [row][mode]
    float *tri_du32 = nullptr;         // Dyy upper diagonal [row] (shared by all modes)
    unsigned char *tri_flag = nullptr; // 1: mode pivots somewhere (FP64 replay)
    int *tri_list = nullptr;           // the flagged modes
    int n_tri_list = 0;
    double *d_tw = nullptr;            // twiddles: x fwd, x bwd, z fwd, z bwd
    int radx[8], nradx, radz[8], nradz;
    // wall model
    double *alpha_x = nullptr, *alpha_z = nullptr, *alpha_zt = nullptr, *tau0 = nullptr;
    double *wtemp1 = nullptr, *wtemp2 = nullptr;   // W at jref: z-interp (nxg,2,nzg), x-interp (nx,2,nzg)
    // learned wall stress (cf_set_wall_mlp): the network, per wall point u_les,
    // stress, envelope flag and the checked eqwm stress; call counter and log
    struct cf_mlp *wmlp = nullptr;
    double *wm_u = nullptr, *wm_tau = nullptr, *wm_tau_eq = nullptr, *wm_log = nullptr;
    int *wm_inside = nullptr, *wm_calls = nullptr;
    int wm_check_every = 0;
    double *eq_grid = nullptr;                      // y_cv(1..ncv), y_fa(1..ncv+1)
    int *eq_zst = nullptr, *eq_xst = nullptr;       // stencil indices
    double *eq_zw = nullptr, *eq_xw = nullptr;      // stencil weights
    int n_nan = 0, n_iter = 0;
    // scalars
    DevScal hs;
    DevScal *ds = nullptr;
    double *d_red = nullptr;           // reduction scratch
    double *d_dtmin = nullptr;         // compute_dt minima per x, y, z index (+inf between calls)
    float2 *d_mass_c = nullptr;        // trapezoid weight of row j as float hi + lo (split path)
    int red_n = 0;
    // staging for transfers
    double *stage = nullptr;
    size_t stage_n = 0;
    // one captured step graph per starting state buffer (the three state
    // buffers rotate with period three)
    cudaGraphExec_t graphs[3] = {};
    int next_buf[3] = {};
    int step_launches = 0;
    int launches = 0;
    bool counting = false;
    // per-kernel timing pass (in_graph: the events are captured into the
    // step's graph as event-record nodes)
    bool profiling = false;
    bool profiling_in_graph = false;
    std::vector<cudaEvent_t> pev;
    std::vector<const char *> pname;
    int pn = 0;
};

int cf_fail(cf_ctx *ctx, int code, const std::string &msg);

// ---- launchers (kernels in the .cu files), all enqueue on ctx->st -------
template <typename T> int launch_bc(cf_ctx *ctx, int buf, bool lo = true);  // apply_boundary_conditions (lo: low words too)
template <typename T> int check_bc(cf_ctx *ctx, int buf, bool *ok);      // ghosts already as the BCs leave them?
template <typename T> int launch_rhs(cf_ctx *ctx, int comp, int slot);     // store F slot
int rhs3_blocks_per_sm(int esz);
template <typename T> int launch_rhs_update(cf_ctx *ctx, int s, int src, int dst);  // fused RHS + RK update
template <typename T> int launch_rk_update(cf_ctx *ctx, int s);            // from stored F slots
template <typename T> int launch_dsm(cf_ctx *ctx, int buf);                // eddy viscosity
template <typename T> int launch_dsm_fused(cf_ctx *ctx, int buf);          // fused pass (periodic state)
template <typename T> int launch_dsm_fused_wm(cf_ctx *ctx, int buf);       // fused pass + seam band (wall model)
int dsm_seam_slots_max();                                                  // partial slots the seam band may take
constexpr int CF_ENS_MAXM = 32;  // channels per batched ensemble launch at most
// fused pass + <LM>/<MM> rows of n channels in two launches (ensembles)
template <typename T> int launch_dsm_batch(cudaStream_t st, cf_ctx *const *m, const int *buf, int n);
// fused right-hand sides + RK update of substep s of n channels in one launch
template <typename T> int launch_rhs3_batch(cudaStream_t st, cf_ctx *const *m, int s, const int *src, const int *dst, int n);
template <typename T> int launch_nut_zero(cf_ctx *ctx);
template <typename T> int launch_nut_materialize(cf_ctx *ctx);       // fill nut if held lazily
template <typename T> int launch_nut_wall_rows(cf_ctx *ctx);         // its rows 1, 2, nyg-1, nyg only (stays lazy)
// canon: project the canonical cells only (the boundary conditions that
// follow rewrite the periodic duplicates)
// one channel's tridiagonal systems for the batched solve of an ensemble
struct TriMember {
    void *spec;                          // spectrum [row][mode], complex of the state's precision
    const double *m, *rd, *du, *dl;      // zgtsv factors [row][mode]
    const unsigned char *piv;
    double2 *scratch;                    // FP64 [row][mode] of the eliminated right-hand side
    int nym, esz;
    long NM, first;                      // modes, first block of the member in the launch
};
TriMember tri_member(const cf_ctx *ctx);
long tri_batch_blocks(long NM);
int launch_tri_batch(cudaStream_t st, const TriMember *dtab, int nmem, long total_blocks);

// Poisson phases (forward transforms, tridiagonal solves, inverse transforms
// and the projection)
enum { POISSON_FWD = 1, POISSON_TRI = 2, POISSON_INV = 4, POISSON_ALL = 7 };
// bc: apply_boundary_conditions after the projection (written by the
// projection kernel itself where it projects canonical cells with no-slip
// walls; launch_bc otherwise)
template <typename T> int launch_projection(cf_ctx *ctx, int buf, bool store_p, bool lo = true, bool canon = false,
                                            int phases = POISSON_ALL, bool bc = false);
template <typename T> int launch_pressure(cf_ctx *ctx, int buf);  // actual pressure into P (pressure.f90:21)
template <typename T> int launch_amd(cf_ctx *ctx, int buf);  // AMD eddy viscosity (subgrid.f90:639)
void amd_plan(int esz, int nxp, int nym, int nzp, int sms, int *nkc, int *nparts);  // z chunks of the AMD pass
int launch_avg_nu_t_flush(cf_ctx *ctx);  // AMD plane means of the last pass, if not formed yet
int amd_partials_for(cf_ctx *ctx, int nkc);  // plane partials per row of an AMD pass with nkc z chunks
constexpr int DSM_ZMAX_HOST = 256;           // planes per z chunk of the fused DSM pass at most
constexpr int RHS_ZMAX_HOST = 256;           // planes per z chunk of the fused RHS at most
template <typename T> int launch_div_check(cf_ctx *ctx, int buf, double *d_out);
template <typename T> int launch_mass_flow(cf_ctx *ctx, int buf, int mode, bool ghosts = false);  // 1: x mass flow, 2: centre-line, 3: y
template <typename T> int launch_mass_value(cf_ctx *ctx, int buf, int mode); // correction into ds->lmax[2] only
template <typename T> int launch_mass_apply(cf_ctx *ctx, int buf, int mode, bool ghosts = false); // add ds->lmax[2], dPdx = it/dt (ghosts: whole array, as the BCs would)
template <typename T> int launch_dt(cf_ctx *ctx, int buf, bool advance_t = false);  // advance_t: t += dt (fast path)
template <typename T> int launch_eqwm(cf_ctx *ctx, int buf);
template <typename T> int launch_wm_inputs(cf_ctx *ctx, int buf, double *ules);  // matching-plane |u| per wall point
int wall_mlp_infer(cf_ctx *ctx, int npts, double h_wm, double nu);  // network stress of every wall point
template <typename T> int launch_copy_state(cf_ctx *ctx, int src, int dst);
template <typename T> int launch_stats(cf_ctx *ctx, int buf, double *d_out);
template <typename T> int launch_monitor(cf_ctx *ctx, int buf, double *d_out);  // (nzg-2) x 8 plane partials

// Called after every kernel launch.  Counts launches while a step is being
// captured, and in a profiling pass records an event after each launch: on
// one stream, launch q runs between event q-1 and event q.
static inline void count_launch(cf_ctx *ctx, const char *name) {
    if (ctx->counting) ctx->launches++;
    if (ctx->profiling) {
        if (ctx->pn < (int)ctx->pev.size()) {
            cudaEventRecordWithFlags(ctx->pev[ctx->pn], ctx->st,
                                     ctx->profiling_in_graph ? cudaEventRecordExternal : cudaEventRecordDefault);
            ctx->pname[ctx->pn] = name;
        }
        ctx->pn++;
    }
}

template <typename T>
static inline RcpT<T> rcp_of(cf_ctx *ctx) {
    const T *b = sizeof(T) == 8 ? (const T *)ctx->d_rgeo : (const T *)ctx->d_rgeo_f;
    RcpT<T> r;
    r.dx = b + ctx->rgeo_off[0];
    r.dxg = b + ctx->rgeo_off[1];
    r.dy = b + ctx->rgeo_off[2];
    r.dyg = b + ctx->rgeo_off[3];
    r.dz = b + ctx->rgeo_off[4];
    r.dzg = b + ctx->rgeo_off[5];
    return r;
}

template <typename T> static inline GeoT<T> geo_of(cf_ctx *ctx);
template <> inline GeoT<double> geo_of<double>(cf_ctx *ctx) { return ctx->geo; }
template <> inline GeoT<float> geo_of<float>(cf_ctx *ctx) { return ctx->geof; }
