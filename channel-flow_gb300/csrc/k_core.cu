// k_core.cu -- boundary conditions, momentum right-hand sides, RK3 update,
// mass-flow forcing, time-step and divergence reductions.
#include <algorithm>


#include "cf_internal.cuh"

// ---------------------------------------------------------------------------
// apply_boundary_conditions (boundary_conditions.f90:20-75).
// One thread per ghost element.  The reference first copies the x-periodic
// planes, then the z-periodic planes (including x ghosts), then overwrites the
// two wall rows for every (i,k); the composed result at a ghost element is
// therefore a copy from the canonical position (wrap(i), j, wrap(k)), and the
// wall rows are built from row 2 / row nyg-1 at (wrap(i), wrap(k)).
// ---------------------------------------------------------------------------
// ybc: 0 = Dirichlet at centres (ghost = -interior), 1 = zero at faces,
//      2 = nonzero Neumann at centres (ghost = interior - dy*alpha(i,wall,k))
struct BcField {
    void *p, *plo;
    int n1, n2, n3, xc, zc, ybc;
    const double *alpha;
    int n;  // ghost elements of this field
};
struct BcSet {
    BcField f[3];
    int nxp, nzp;
    double dyb, dyt;
};

template <typename T>
__device__ __forceinline__ void bc_elem(const BcField &d, int nxp, int nzp, double dyb, double dyt, int t) {
    const Fld<T> F = make_fld<T>(d.p, d.n1, d.n2), Flo = make_fld<T>(d.plo, d.n1, d.n2);
    const int n1 = d.n1, n2 = d.n2, n3 = d.n3, xc = d.xc, zc = d.zc, ybc = d.ybc;
    const int gx = xc ? 3 : 2, gz = zc ? 3 : 2;
    const int nY = 2 * n1 * n3;
    const int nX = gx * (n2 - 2) * n3;
    int i, j, k;
    if (t < nY) {
        i = t % n1 + 1;
        int r = t / n1;
        k = r % n3 + 1;
        j = (r / n3) == 0 ? 1 : n2;
        int is = wrapc(i, nxp), ks = wrapc(k, nzp);
        if (ybc == 1) {
            F(i, j, k) = T(0);
            if (Flo.p) Flo(i, j, k) = T(0);
        } else {
            int jsrc = (j == 1) ? 2 : n2 - 1;
            T v = F(is, jsrc, ks);
            if (ybc == 0) {
                F(i, j, k) = -v;
                if (Flo.p) Flo(i, j, k) = -Flo(is, jsrc, ks);
            } else {
                int w = (j == 1) ? 0 : 1;
                double a = d.alpha[(i - 1) + (long)n1 * (w + 2L * (k - 1))];
                double dy = (j == 1) ? dyb : dyt;
                if (Flo.p) {
                    double hv = (double)v + (double)Flo(is, jsrc, ks) - dy * a;
                    T hi = (T)hv;
                    F(i, j, k) = hi;
                    Flo(i, j, k) = (T)(hv - (double)hi);
                } else {
                    F(i, j, k) = (T)((double)v - dy * a);
                }
            }
        }
        return;
    }
    t -= nY;
    if (t < nX) {
        int g = t % gx;
        int r = t / gx;
        j = r % (n2 - 2) + 2;
        k = r / (n2 - 2) + 1;
        i = (g == 0) ? 1 : (xc ? (g == 1 ? n1 - 1 : n1) : n1);
    } else {
        t -= nX;
        int g = t % gz;
        int r = t / gz;
        j = r % (n2 - 2) + 2;
        i = r / (n2 - 2) + 2;  // non-ghost x: 2 .. n1-gx+1
        k = (g == 0) ? 1 : (zc ? (g == 1 ? n3 - 1 : n3) : n3);
    }
    int is = wrapc(i, nxp), ks = wrapc(k, nzp);
    F(i, j, k) = F(is, j, ks);
    if (Flo.p) Flo(i, j, k) = Flo(is, j, ks);
}

// The ghost shells of U, V and W in one launch: thread t belongs to the
// field whose element range contains it.
template <typename T>
__global__ void k_bc(BcSet s) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        if (t < s.f[q].n) {
            bc_elem<T>(s.f[q], s.nxp, s.nzp, s.dyb, s.dyt, t);
            return;
        }
        t -= s.f[q].n;
    }
}

// Whether the ghosts already hold what apply_boundary_conditions would put
// there (no-slip walls): element t of the same enumeration as k_bc compared
// with its source; any mismatch sets *bad.
template <typename T>
__device__ __forceinline__ bool bc_elem_ok(const BcField &d, int nxp, int nzp, int t) {
    const Fld<T> F = make_fld<T>(d.p, d.n1, d.n2), Flo = make_fld<T>(d.plo, d.n1, d.n2);
    const int n1 = d.n1, n2 = d.n2, n3 = d.n3, xc = d.xc, zc = d.zc, ybc = d.ybc;
    const int gx = xc ? 3 : 2, gz = zc ? 3 : 2;
    const int nY = 2 * n1 * n3, nX = gx * (n2 - 2) * n3;
    int i, j, k;
    if (t < nY) {
        i = t % n1 + 1;
        const int r = t / n1;
        k = r % n3 + 1;
        j = (r / n3) == 0 ? 1 : n2;
        const int is = wrapc(i, nxp), ks = wrapc(k, nzp), jsrc = (j == 1) ? 2 : n2 - 1;
        if (ybc == 1) return F(i, j, k) == T(0) && (!Flo.p || Flo(i, j, k) == T(0));
        return F(i, j, k) == -F(is, jsrc, ks) && (!Flo.p || Flo(i, j, k) == -Flo(is, jsrc, ks));
    }
    t -= nY;
    if (t < nX) {
        const int g = t % gx, r = t / gx;
        j = r % (n2 - 2) + 2;
        k = r / (n2 - 2) + 1;
        i = (g == 0) ? 1 : (xc ? (g == 1 ? n1 - 1 : n1) : n1);
    } else {
        t -= nX;
        const int g = t % gz, r = t / gz;
        j = r % (n2 - 2) + 2;
        i = r / (n2 - 2) + 2;
        k = (g == 0) ? 1 : (zc ? (g == 1 ? n3 - 1 : n3) : n3);
    }
    const int is = wrapc(i, nxp), ks = wrapc(k, nzp);
    return F(i, j, k) == F(is, j, ks) && (!Flo.p || Flo(i, j, k) == Flo(is, j, ks));
}

template <typename T>
__global__ void k_bc_check(BcSet s, int *bad) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        if (t < s.f[q].n) {
            if (!bc_elem_ok<T>(s.f[q], s.nxp, s.nzp, t)) atomicOr(bad, 1);
            return;
        }
        t -= s.f[q].n;
    }
}

static BcField bc_field(void *p, void *plo, int n1, int n2, int n3, int xc, int zc, int ybc, const double *alpha) {
    BcField f;
    int gx = xc ? 3 : 2, gz = zc ? 3 : 2;
    f.p = p;
    f.plo = plo;
    f.n1 = n1;
    f.n2 = n2;
    f.n3 = n3;
    f.xc = xc;
    f.zc = zc;
    f.ybc = ybc;
    f.alpha = alpha;
    f.n = 2 * n1 * n3 + gx * (n2 - 2) * n3 + gz * (n2 - 2) * (n1 - gx);
    return f;
}

template <typename T>
int launch_bc(cf_ctx *ctx, int b, bool lo) {
    int wm = ctx->prm.iwall_model;
    ctx->state_periodic = true;  // holds for every later launch on the stream
    BcSet s;
    // U: x faces, y centres, z centres
    s.f[0] = bc_field(ctx->U[b], lo ? ctx->Ulo[b] : nullptr, ctx->nx, ctx->nyg, ctx->nzg, 0, 1, wm == 3 ? 2 : 0, ctx->alpha_x);
    // V: x centres, y faces, z centres
    s.f[1] = bc_field(ctx->V[b], lo ? ctx->Vlo[b] : nullptr, ctx->nxg, ctx->ny, ctx->nzg, 1, 1, 1, nullptr);
    // W: x centres, y centres, z faces
    s.f[2] = bc_field(ctx->W[b], lo ? ctx->Wlo[b] : nullptr, ctx->nxg, ctx->nyg, ctx->nz, 1, 0, wm == 3 ? 2 : 0, ctx->alpha_z);
    s.nxp = ctx->nxp;
    s.nzp = ctx->nzp;
    s.dyb = ctx->hyg[2] - ctx->hyg[1];
    s.dyt = ctx->hyg[ctx->nyg] - ctx->hyg[ctx->nyg - 1];
    const int tot = s.f[0].n + s.f[1].n + s.f[2].n;
    k_bc<T><<<cdiv(tot, 256), 256, 0, ctx->st>>>(s);
    count_launch(ctx, "k_bc");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// Momentum right-hand sides, equations.f90:24-498, one thread per point.
// ---------------------------------------------------------------------------
struct RkCoef {
    double c[4][4];
};

// The spacings enter as reciprocals (rc): 1/(xg(i+1)-xg(i)) = rc.dxg[i+1],
// 1/(x(i)-x(i-1)) = rc.dx[i], and so on.
//
// ZC (the z-marching fused kernel): the z-face terms of a cell -- its
// advective and viscous fluxes through the faces k-1/2 and k+1/2 -- are
// taken as rdz3 * (F(k+1/2) - F(k-1/2)) with F = viscous flux less advective
// flux; *fz holds F(k-1/2) on entry (carried from the cell below, or formed
// by rhs_*_zflux_dn for the first plane of a chunk) and F(k+1/2) as the
// next cell's F(k-1/2) on return (for u with the spacing 1/(x(i)-x(i-1))
// that the reference's lower face uses, rdx1; the cell's own upper face
// uses rdx2).
template <typename T, typename A, typename RC, bool ZC = false>
__device__ __forceinline__ T rhs_u_point(const GeoT<T> &g, const RC &rc, const A &U, const A &V, const A &W,
                                         const A &nt, T nu, T dPdx, T Om, bool rot, int i, int j, int k,
                                         T *fz = nullptr) {
    const T *w0 = g.w0, *w1 = g.w1;
    const T h = T(0.5), q = T(0.25);
    const T rdx1 = rc.dx[i], rdx2 = rc.dx[i + 1], rdx3 = rc.dxg[i + 1];
    const T rdy3 = rc.dy[j];
    const T rdz1 = rc.dzg[k], rdz2 = rc.dzg[k + 1], rdz3 = rc.dz[k];
    // 1) -du^2/dx  (equations.f90:43-57)
    T a = h * (U(i, j, k) + U(i + 1, j, k));
    T b = h * (U(i - 1, j, k) + U(i, j, k));
    T r = -(a * a - b * b) * rdx3;
    // 2) -duv/dy   (:62-79)
    T uy1 = w0[j] * U(i, j, k) + w1[j] * U(i, j + 1, k);
    T uy0 = w0[j - 1] * U(i, j - 1, k) + w1[j - 1] * U(i, j, k);
    T vx1 = h * (V(i, j, k) + V(i + 1, j, k));
    T vx0 = h * (V(i, j - 1, k) + V(i + 1, j - 1, k));
    r += -(uy1 * vx1 - uy0 * vx0) * rdy3;
    // 3) -duw/dz   (:84-101)
    T uz1 = h * (U(i, j, k) + U(i, j, k + 1));
    T wx1 = h * (W(i, j, k) + W(i + 1, j, k));
    if constexpr (!ZC) {
        T uz0 = h * (U(i, j, k - 1) + U(i, j, k));
        T wx0 = h * (W(i, j, k - 1) + W(i + 1, j, k - 1));
        r += -(uz1 * wx1 - uz0 * wx0) * rdz3;
    }
    // 4) viscous   (:108-163)
    T t2j = (U(i, j + 1, k) - U(i, j, k)) * rc.dyg[j + 1];
    T t2jm = (U(i, j, k) - U(i, j - 1, k)) * rc.dyg[j];
    T nu_x1 = nu + nt(i, j, k);
    T nu_x2 = nu + nt(i + 1, j, k);
    T nu_y1 = nu + h * (w0[j - 1] * nt(i, j - 1, k) + w1[j - 1] * nt(i, j, k) + w0[j - 1] * nt(i + 1, j - 1, k) +
                        w1[j - 1] * nt(i + 1, j, k));
    T nu_y2 = nu + h * (w0[j] * nt(i, j, k) + w1[j] * nt(i, j + 1, k) + w0[j] * nt(i + 1, j, k) + w1[j] * nt(i + 1, j + 1, k));
    T nu_z2 = nu + q * (nt(i, j, k) + nt(i, j, k + 1) + nt(i + 1, j, k) + nt(i + 1, j, k + 1));
    T visc = T(2) * rdx3 * (nu_x2 * (U(i + 1, j, k) - U(i, j, k)) * rdx2 - nu_x1 * (U(i, j, k) - U(i - 1, j, k)) * rdx1) +
             rdy3 * (nu_y2 * (t2j + (V(i + 1, j, k) - V(i, j, k)) * rdx2) -
                     nu_y1 * (t2jm + (V(i + 1, j - 1, k) - V(i, j - 1, k)) * rdx1));
    if constexpr (!ZC) {
        T nu_z1 = nu + q * (nt(i, j, k) + nt(i, j, k - 1) + nt(i + 1, j, k) + nt(i + 1, j, k - 1));
        visc += rdz3 * (nu_z2 * ((U(i, j, k + 1) - U(i, j, k)) * rdz2 + (W(i + 1, j, k) - W(i, j, k)) * rdx2) -
                        nu_z1 * ((U(i, j, k) - U(i, j, k - 1)) * rdz1 + (W(i + 1, j, k - 1) - W(i, j, k - 1)) * rdx1));
        r += visc;
    } else {
        r += visc;
        const T gz = (U(i, j, k + 1) - U(i, j, k)) * rdz2, dw = W(i + 1, j, k) - W(i, j, k), a = uz1 * wx1;
        r += rdz3 * ((nu_z2 * (gz + dw * rdx2) - a) - *fz);
        *fz = nu_z2 * (gz + dw * rdx1) - a;
    }
    r += dPdx;  // :166
    if (rot) {  // |Om| > 1e-6, :169-177
        T tv0 = h * (V(i, j - 1, k) + V(i, j, k));
        T tv1 = h * (V(i + 1, j - 1, k) + V(i + 1, j, k));
        r += T(2) * Om * (h * (tv0 + tv1));
    }
    return r;
}

template <typename T, typename A, typename RC, bool ZC = false>
__device__ __forceinline__ T rhs_v_point(const GeoT<T> &g, const RC &rc, const A &U, const A &V, const A &W,
                                         const A &nt, T nu, T Om, bool rot, int i, int j, int k, T *fz = nullptr) {
    const T *w0 = g.w0, *w1 = g.w1;
    const T h = T(0.5);
    const T rdx1 = rc.dxg[i], rdx2 = rc.dxg[i + 1], rdx3 = rc.dx[i];
    const T rdy1 = rc.dy[j], rdy2 = rc.dy[j + 1], rdy3 = rc.dyg[j + 1];
    const T rdz1 = rc.dzg[k], rdz2 = rc.dzg[k + 1], rdz3 = rc.dz[k];
    // 1) -dv^2/dy (equations.f90:205-223)
    T a = h * (V(i, j, k) + V(i, j + 1, k));
    T b = h * (V(i, j - 1, k) + V(i, j, k));
    T r = -(a * a - b * b) * rdy3;
    // 2) -duv/dx (:228-245)
    T uy1 = w0[j] * U(i, j, k) + w1[j] * U(i, j + 1, k);
    T uy0 = w0[j] * U(i - 1, j, k) + w1[j] * U(i - 1, j + 1, k);
    T vx1 = h * (V(i, j, k) + V(i + 1, j, k));
    T vx0 = h * (V(i - 1, j, k) + V(i, j, k));
    r += -(uy1 * vx1 - uy0 * vx0) * rdx3;
    // 3) -dvw/dz (:250-267)
    T vz1 = h * (V(i, j, k) + V(i, j, k + 1));
    T wy1 = w0[j] * W(i, j, k) + w1[j] * W(i, j + 1, k);
    if constexpr (!ZC) {
        T vz0 = h * (V(i, j, k - 1) + V(i, j, k));
        T wy0 = w0[j] * W(i, j, k - 1) + w1[j] * W(i, j + 1, k - 1);
        r += -(vz1 * wy1 - vz0 * wy0) * rdz3;
    }
    // 4) viscous (:276-331)
    T nu_x1 = nu + h * (w0[j] * nt(i - 1, j, k) + w1[j] * nt(i - 1, j + 1, k) + w0[j] * nt(i, j, k) + w1[j] * nt(i, j + 1, k));
    T nu_x2 = nu + h * (w0[j] * nt(i, j, k) + w1[j] * nt(i, j + 1, k) + w0[j] * nt(i + 1, j, k) + w1[j] * nt(i + 1, j + 1, k));
    T nu_y1 = nu + nt(i, j, k);
    T nu_y2 = nu + nt(i, j + 1, k);
    T nu_z2 = nu + h * (w0[j] * nt(i, j, k) + w1[j] * nt(i, j + 1, k) + w0[j] * nt(i, j, k + 1) + w1[j] * nt(i, j + 1, k + 1));
    T visc = rdx3 * (nu_x2 * ((V(i + 1, j, k) - V(i, j, k)) * rdx2 + (U(i, j + 1, k) - U(i, j, k)) * rdy3) -
                     nu_x1 * ((V(i, j, k) - V(i - 1, j, k)) * rdx1 + (U(i - 1, j + 1, k) - U(i - 1, j, k)) * rdy3)) +
             T(2) * rdy3 * (nu_y2 * (V(i, j + 1, k) - V(i, j, k)) * rdy2 - nu_y1 * (V(i, j, k) - V(i, j - 1, k)) * rdy1);
    if constexpr (!ZC) {
        T nu_z1 = nu + h * (w0[j] * nt(i, j, k - 1) + w1[j] * nt(i, j + 1, k - 1) + w0[j] * nt(i, j, k) + w1[j] * nt(i, j + 1, k));
        visc += rdz3 * (nu_z2 * ((V(i, j, k + 1) - V(i, j, k)) * rdz2 + (W(i, j + 1, k) - W(i, j, k)) * rdy3) -
                        nu_z1 * ((V(i, j, k) - V(i, j, k - 1)) * rdz1 + (W(i, j + 1, k - 1) - W(i, j, k - 1)) * rdy3));
        r += visc;
    } else {
        r += visc;
        const T f = nu_z2 * ((V(i, j, k + 1) - V(i, j, k)) * rdz2 + (W(i, j + 1, k) - W(i, j, k)) * rdy3) - vz1 * wy1;
        r += rdz3 * (f - *fz);
        *fz = f;
    }
    if (rot) {  // :334-342
        T tu0 = h * (U(i - 1, j, k) + U(i, j, k));
        T tu1 = h * (U(i - 1, j + 1, k) + U(i, j + 1, k));
        r -= T(2) * Om * (w0[j] * tu0 + w1[j] * tu1);
    }
    return r;
}

template <typename T, typename A, typename RC, bool ZC = false>
__device__ __forceinline__ T rhs_w_point(const GeoT<T> &g, const RC &rc, const A &U, const A &V, const A &W,
                                         const A &nt, T nu, T dPdz, int i, int j, int k, T *fz = nullptr) {
    const T *w0 = g.w0, *w1 = g.w1;
    const T h = T(0.5), q = T(0.25);
    const T rdx1 = rc.dxg[i], rdx2 = rc.dxg[i + 1], rdx3 = rc.dx[i];
    const T rdy3 = rc.dy[j];
    const T rdz1 = rc.dz[k], rdz2 = rc.dz[k + 1], rdz3 = rc.dzg[k + 1];
    // 1) -dw^2/dz (equations.f90:370-384)
    T a = h * (W(i, j, k) + W(i, j, k + 1));
    T r = T(0);
    if constexpr (!ZC) {
        T b = h * (W(i, j, k - 1) + W(i, j, k));
        r = -(a * a - b * b) * rdz3;
    }
    // 2) -duw/dx (:389-406)
    T uz1 = h * (U(i, j, k) + U(i, j, k + 1));
    T uz0 = h * (U(i - 1, j, k) + U(i - 1, j, k + 1));
    T wx1 = h * (W(i, j, k) + W(i + 1, j, k));
    T wx0 = h * (W(i - 1, j, k) + W(i, j, k));
    r += -(uz1 * wx1 - uz0 * wx0) * rdx3;
    // 3) -dvw/dy (:411-428)
    T vz1 = h * (V(i, j, k) + V(i, j, k + 1));
    T vz0 = h * (V(i, j - 1, k) + V(i, j - 1, k + 1));
    T wy1 = w0[j] * W(i, j, k) + w1[j] * W(i, j + 1, k);
    T wy0 = w0[j - 1] * W(i, j - 1, k) + w1[j - 1] * W(i, j, k);
    r += -(vz1 * wy1 - vz0 * wy0) * rdy3;
    // 4) viscous (:435-493)
    T t2j = (W(i, j + 1, k) - W(i, j, k)) * rc.dyg[j + 1];
    T t2jm = (W(i, j, k) - W(i, j - 1, k)) * rc.dyg[j];
    T nu_x1 = nu + q * (nt(i, j, k) + nt(i, j, k + 1) + nt(i - 1, j, k) + nt(i - 1, j, k + 1));
    T nu_x2 = nu + q * (nt(i, j, k) + nt(i, j, k + 1) + nt(i + 1, j, k) + nt(i + 1, j, k + 1));
    T nu_y1 = nu + h * (w0[j - 1] * nt(i, j - 1, k) + w1[j - 1] * nt(i, j, k) + w0[j - 1] * nt(i, j - 1, k + 1) +
                        w1[j - 1] * nt(i, j, k + 1));
    T nu_y2 = nu + h * (w0[j] * nt(i, j, k) + w1[j] * nt(i, j + 1, k) + w0[j] * nt(i, j, k + 1) + w1[j] * nt(i, j + 1, k + 1));
    T nu_z2 = nu + nt(i, j, k + 1);
    T visc = rdx3 * (nu_x2 * ((W(i + 1, j, k) - W(i, j, k)) * rdx2 + (U(i, j, k + 1) - U(i, j, k)) * rdz2) -
                     nu_x1 * ((W(i, j, k) - W(i - 1, j, k)) * rdx1 + (U(i - 1, j, k + 1) - U(i - 1, j, k)) * rdz1)) +
             rdy3 * (nu_y2 * (t2j + (V(i, j, k + 1) - V(i, j, k)) * rdz2) -
                     nu_y1 * (t2jm + (V(i, j - 1, k + 1) - V(i, j - 1, k)) * rdz1));
    if constexpr (!ZC) {
        T nu_z1 = nu + nt(i, j, k);
        visc += T(2) * rdz3 * (nu_z2 * (W(i, j, k + 1) - W(i, j, k)) * rdz2 - nu_z1 * (W(i, j, k) - W(i, j, k - 1)) * rdz1);
        r += visc;
    } else {
        r += visc;
        const T f = T(2) * (nu_z2 * (W(i, j, k + 1) - W(i, j, k)) * rdz2) - a * a;
        r += rdz3 * (f - *fz);
        *fz = f;
    }
    r += dPdz;  // :496
    return r;
}

// F(k-1/2) of the u, v and w cells at (i, j, k) as the reference's lower
// z faces take them (the first plane of a z-marching chunk; later planes
// carry it from the cell below, see ZC above).
template <typename T, typename A, typename RC>
__device__ __forceinline__ void rhs_zflux_dn(const GeoT<T> &g, const RC &rc, const A &U, const A &V, const A &W,
                                             const A &nt, T nu, int i, int j, int k, T &fu, T &fv, T &fw) {
    const T *w0 = g.w0, *w1 = g.w1;
    const T h = T(0.5), q = T(0.25);
    {
        const T uz0 = h * (U(i, j, k - 1) + U(i, j, k)), wx0 = h * (W(i, j, k - 1) + W(i + 1, j, k - 1));
        const T nu_z1 = nu + q * (nt(i, j, k) + nt(i, j, k - 1) + nt(i + 1, j, k) + nt(i + 1, j, k - 1));
        fu = nu_z1 * ((U(i, j, k) - U(i, j, k - 1)) * rc.dzg[k] + (W(i + 1, j, k - 1) - W(i, j, k - 1)) * rc.dx[i]) -
             uz0 * wx0;
    }
    {
        const T vz0 = h * (V(i, j, k - 1) + V(i, j, k)), wy0 = w0[j] * W(i, j, k - 1) + w1[j] * W(i, j + 1, k - 1);
        const T nu_z1 =
            nu + h * (w0[j] * nt(i, j, k - 1) + w1[j] * nt(i, j + 1, k - 1) + w0[j] * nt(i, j, k) + w1[j] * nt(i, j + 1, k));
        fv = nu_z1 * ((V(i, j, k) - V(i, j, k - 1)) * rc.dzg[k] + (W(i, j + 1, k - 1) - W(i, j, k - 1)) * rc.dyg[j + 1]) -
             vz0 * wy0;
    }
    {
        const T b = h * (W(i, j, k - 1) + W(i, j, k));
        const T nu_z1 = nu + nt(i, j, k);
        fw = T(2) * (nu_z1 * (W(i, j, k) - W(i, j, k - 1)) * rc.dz[k]) - b * b;
    }
}

// RK3 stage update of one point (time_integration.f90:108-110, 124-126,
// 140-145) with F2 never reused (rk_coef(3,2) = 0, initialization.f90:416).
// The split path keeps u^n as hi + lo; substep 3 writes the new low word.
template <typename T>
__device__ __forceinline__ void rk_store(T r, int i, int j, int k, const Fld<T> &out, const Fld<T> &F1,
                                         const Fld<T> &Uo, const Fld<T> &Uolo, const Fld<T> &Unlo, int s,
                                         const RkCoef &rk, T dt) {
    T inc;
    if (s == 1) {
        F1(i, j, k) = r;
        inc = dt * T(rk.c[1][1]) * r;
    } else if (s == 2) {
        inc = dt * (T(rk.c[2][1]) * F1(i, j, k) + T(rk.c[2][2]) * r);
    } else {
        inc = dt * (T(rk.c[3][1]) * F1(i, j, k) + T(rk.c[3][3]) * r);
    }
    if constexpr (sizeof(T) == 4) {
        if (Uolo.p) {
            float hi = Uo(i, j, k), lo = Uolo(i, j, k);
            if (Unlo.p) {
                ff_add(hi, lo, inc);
                out(i, j, k) = hi;
                Unlo(i, j, k) = lo;
            } else {
                out(i, j, k) = hi + (lo + inc);
            }
            return;
        }
    }
    out(i, j, k) = Uo(i, j, k) + inc;
}

// The same update with its operands already loaded (f1 = F1 for s > 1, uo and
// uolo = the old state and its low word) and the substep's coefficients in T
// (ca: of F1 -- or of r when s = 1 --, cb: of r).
template <typename T>
__device__ __forceinline__ void rk_apply(T r, T f1, T uo, T uolo, bool has_lo, int i, int j, int k, const Fld<T> &out,
                                         const Fld<T> &F1, const Fld<T> &Unlo, int s, T ca, T cb, T dt) {
    T inc;
    if (s == 1) {
        F1(i, j, k) = r;
        inc = dt * ca * r;
    } else {
        inc = dt * (ca * f1 + cb * r);
    }
    if constexpr (sizeof(T) == 4) {
        if (has_lo) {
            float hi = uo, lo = uolo;
            if (Unlo.p) {
                ff_add(hi, lo, inc);
                out(i, j, k) = hi;
                Unlo(i, j, k) = lo;
            } else {
                out(i, j, k) = hi + (lo + inc);
            }
            return;
        }
    }
    out(i, j, k) = uo + inc;
}

// mode: 0 = store F(slot); 1 = fused update from Uo with F1 (s = 1 stores F1)
template <typename T, int COMP>
__global__ void k_rhs(GeoT<T> g, RcpT<T> rc, Fld<T> U, Fld<T> V, Fld<T> W, Fld<T> nt, const DevScal *ds, T nu, T Om, int rot,
                      Fld<T> out, Fld<T> F1, Fld<T> Uo, Fld<T> Uolo, Fld<T> Unlo, int mode, int s, RkCoef rk,
                      int i1, int j1, int k1) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
    int k = blockIdx.z + 2;
    if (i > i1 || j > j1 || k > k1) return;
    T r;
    if (COMP == 0) r = rhs_u_point<T, Fld<T>>(g, rc, U, V, W, nt, nu, ds_dpdx<T>(ds), Om, rot, i, j, k);
    else if (COMP == 1) r = rhs_v_point<T, Fld<T>>(g, rc, U, V, W, nt, nu, Om, rot, i, j, k);
    else r = rhs_w_point<T, Fld<T>>(g, rc, U, V, W, nt, nu, ds_dpdz<T>(ds), i, j, k);
    if (mode == 0) {
        out(i, j, k) = r;
        return;
    }
    rk_store<T>(r, i, j, k, out, F1, Uo, Uolo, Unlo, s, rk, ds_dt<T>(ds));
}


static RkCoef rk_coefs() {
    RkCoef c = {};
    c.c[1][1] = 8.0 / 15.0;
    c.c[2][1] = 1.0 / 4.0;
    c.c[2][2] = 5.0 / 12.0;
    c.c[3][1] = 1.0 / 4.0;
    c.c[3][2] = 0.0;
    c.c[3][3] = 3.0 / 4.0;
    return c;
}

template <typename T>
static int rhs_launch(cf_ctx *ctx, int comp, int src, int mode, int s, int slot, int dst) {
    if (int rc = launch_nut_materialize<T>(ctx)) return rc;
    GeoT<T> g = geo_of<T>(ctx);
    Fld<T> U = make_fld<T>(ctx->U[src], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[src], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[src], ctx->nxg, ctx->nyg);
    Fld<T> nt = make_fld<T>(ctx->nut, ctx->nxg, ctx->nyg);
    int i1, j1, k1, n1, n2;
    void *outp, *uo, *uolo = nullptr, *unlo = nullptr;
    if (comp == 0) { i1 = ctx->nx - 1; j1 = ctx->nyg - 1; k1 = ctx->nzg - 1; n1 = ctx->nx; n2 = ctx->nyg; }
    else if (comp == 1) { i1 = ctx->nxg - 1; j1 = ctx->ny - 1; k1 = ctx->nzg - 1; n1 = ctx->nxg; n2 = ctx->ny; }
    else { i1 = ctx->nxg - 1; j1 = ctx->nyg - 1; k1 = ctx->nz - 1; n1 = ctx->nxg; n2 = ctx->nyg; }
    void **cur = comp == 0 ? ctx->U : comp == 1 ? ctx->V : ctx->W;
    void **lo = comp == 0 ? ctx->Ulo : comp == 1 ? ctx->Vlo : ctx->Wlo;
    if (mode == 0) {
        outp = ctx->F[slot][comp];
        uo = nullptr;
    } else {
        outp = cur[dst];
        uo = cur[ctx->old];
        if (lo[ctx->old]) {
            uolo = lo[ctx->old];
            if (s == 3) unlo = lo[dst];
        }
    }
    // F arrays use the full field extents (interior written)
    Fld<T> out = make_fld<T>(outp, n1, n2);
    Fld<T> F1 = make_fld<T>(ctx->F[0][comp], n1, n2);
    Fld<T> Uo = make_fld<T>(uo, n1, n2);
    Fld<T> Uolo = make_fld<T>(uolo, n1, n2);
    Fld<T> Unlo = make_fld<T>(unlo, n1, n2);
    dim3 blk(32, 4, 1), grd(cdiv(i1 - 1, 32), cdiv(j1 - 1, 4), k1 - 1);
    T nu = (T)ctx->prm.nu, Om = (T)ctx->omega_z;
    const int rot = fabs(ctx->omega_z) > 1e-6;  // equations.f90:169, 334
    RkCoef rk = rk_coefs();
    if (comp == 0) k_rhs<T, 0><<<grd, blk, 0, ctx->st>>>(g, rcp_of<T>(ctx), U, V, W, nt, ctx->ds, nu, Om, rot, out, F1, Uo, Uolo, Unlo, mode, s, rk, i1, j1, k1);
    else if (comp == 1) k_rhs<T, 1><<<grd, blk, 0, ctx->st>>>(g, rcp_of<T>(ctx), U, V, W, nt, ctx->ds, nu, Om, rot, out, F1, Uo, Uolo, Unlo, mode, s, rk, i1, j1, k1);
    else k_rhs<T, 2><<<grd, blk, 0, ctx->st>>>(g, rcp_of<T>(ctx), U, V, W, nt, ctx->ds, nu, Om, rot, out, F1, Uo, Uolo, Unlo, mode, s, rk, i1, j1, k1);
    count_launch(ctx, "k_rhs");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// Fused right-hand sides of u, v and w with the RK update, one launch per
// substep.  A block owns a TX x TY tile of (i, j) columns and marches along z
// over a chunk of planes, keeping planes k-1, k, k+1 of U, V, W and nu_t (tile
// plus one halo cell) in a shared-memory ring; the per-point formulas above
// read them through an accessor with the Fld interface.
// ---------------------------------------------------------------------------
template <typename T, int TX, int TY>
struct RingAcc {
    static constexpr int SX = TX + 2, SY = TY + 2;
    const T *b[3];  // planes k-1, k, k+1 of one field
    int i0, j0, kc;
    __device__ __forceinline__ T operator()(int i, int j, int k) const {
        return b[k - kc + 1][(j - j0 + 1) * SX + (i - i0 + 1)];
    }
};

template <typename T>
struct Trio {
    Fld<T> u, v, w;
};

// nu_t held as |S| on canonical cells and the plane coefficient C(j):
// nu_t(i,j,k) = max(-C(jj)|S|(wrap i, jj, wrap k)/2, 0), jj = j clamped to
// the interior, negated on the wall ghost rows for Dirichlet_nu_t
// (subgrid.f90:521-536).  S == nullptr: read the nut field instead.
template <typename T>
struct NutSrc {
    const T *S;
    const T *C;  // 1-based rows
    int nxp, nym, nzp, dirichlet;
};

// planes per z chunk of the fused RHS (its z spacings sit in shared memory)
constexpr int RHS_ZMAX = RHS_ZMAX_HOST;
// resident blocks per SM the fused RHS is compiled for.  With u, v and w
// computed before any store, the shared-memory reads common to them are
// issued once but more values stay live; with the per-thread index and mask
// set-up hoisted out of the march and the substep and low words compile-time,
// the FP32 kernel fits three blocks of 256 threads (85 registers): 24 warps
// per SM instead of 16, 133 -> 105 us per launch at Re_tau 550.  FP64 keeps two.
template <typename T> struct RhsMinB { static constexpr int v = sizeof(T) == 4 ? 3 : 2; };

// Everything one launch of the fused right-hand side needs for one channel
// (the grid of blocks is ntx x nty x nkc).
template <typename T>
struct Rhs3Args {
    GeoT<T> g;
    RcpT<T> rc;
    Fld<T> U, V, W, nt;
    NutSrc<T> ns;
    const DevScal *ds;
    T nu, Om, ca, cb;
    int rot, s, kc_len, ilim, klim, ntx, nty, nkc;
    Trio<T> out, F1, Uo, Uolo, Unlo;
};

// The RK update of one point for substep S (time_integration.f90:108-145):
// S = 1 stores the right-hand side as F1; LO: the split path's low words
// (u^n = hi + lo; substep 3 stores the new state as hi + lo, the others the
// rounded sum).  o: the point's index, the same in every field of its
// component.
template <typename T, int S, bool LO>
__device__ __forceinline__ void rk_apply_at(T r, T f1, T uo, T uolo, int o, T *out, T *F1, T *Unlo, T ca, T cb, T dt) {
    T inc;
    if constexpr (S == 1) {
        F1[o] = r;
        inc = dt * ca * r;
    } else {
        inc = dt * (ca * f1 + cb * r);
    }
    if constexpr (sizeof(T) == 4 && LO) {
        float hi = uo, lo = uolo;
        if constexpr (S == 3) {
            ff_add(hi, lo, inc);
            out[o] = hi;
            Unlo[o] = lo;
        } else {
            out[o] = hi + (lo + inc);
        }
    } else {
        out[o] = uo + inc;
    }
}

// The tile (bx, by, bz) of one channel: a block of the single-channel launch
// or of the ensemble launch (k_rhs3_batch below), for substep S (LO: low
// words of u^n present).  Every per-point index is formed once per thread
// (the (i, j) part, planes follow by adding the plane stride), the ring's
// loads are predicated by masks fixed for the march.
template <typename T, int TX, int TY, int S, bool LO>
__device__ __forceinline__ void rhs3_tile(const Rhs3Args<T> &args, int bx, int by, int bz) {
    const GeoT<T> g = args.g;
    const RcpT<T> rc = args.rc;
    const Fld<T> U = args.U, V = args.V, W = args.W, nt = args.nt;
    const NutSrc<T> ns = args.ns;
    const DevScal *const ds = args.ds;
    const T nu = args.nu, Om = args.Om, ca = args.ca, cb = args.cb;
    const int rot = args.rot, kc_len = args.kc_len, ilim = args.ilim, klim = args.klim;
    const Trio<T> out = args.out, F1 = args.F1, Uo = args.Uo, Uolo = args.Uolo, Unlo = args.Unlo;
    constexpr int SX = TX + 2, SY = TY + 2, NP = SX * SY, NT = TX * TY, NL = (NP + NT - 1) / NT;
    __shared__ T ring[3][4][NP];  // [plane slot][field U V W nu_t][tile]
    const int nx = g.nx, ny = g.ny, nz = g.nz, nxg = g.nxg, nyg = g.nyg, nzg = g.nzg;
    const int i0 = 2 + bx * TX, j0 = 2 + by * TY;
    const int kb = 2 + bz * kc_len, ke = min(kb + kc_len - 1, klim);
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int i = i0 + tx, j = j0 + ty;
    const T dt = ds_dt<T>(ds), dPdx = ds_dpdx<T>(ds), dPdz = ds_dpdz<T>(ds);
    // the tile's x and y reciprocal spacings and interpolation weights, and
    // the chunk's z reciprocal spacings, in shared memory; gl and rcs index
    // them with the global 1-based indices
    __shared__ T gxs[2][TX + 3], gys[4][TY + 3], gzs[2][RHS_ZMAX + 2];
    for (int t = threadIdx.x; t < TX + 3; t += TX * TY) {
        const int ii = i0 - 1 + t;
        gxs[0][t] = rc.dx[min(ii, nx + 1)];
        gxs[1][t] = rc.dxg[min(ii, nxg + 1)];
    }
    for (int t = threadIdx.x; t < TY + 3; t += TX * TY) {
        const int jj = j0 - 1 + t;
        gys[0][t] = rc.dy[min(jj, ny + 1)];
        gys[1][t] = rc.dyg[min(jj, nyg + 1)];
        gys[2][t] = g.w0[min(jj, ny)];
        gys[3][t] = g.w1[min(jj, ny)];
    }
    for (int t = threadIdx.x; t < ke - kb + 2; t += TX * TY) {
        const int kk = kb + t;
        gzs[0][t] = rc.dz[min(kk, nz + 1)];
        gzs[1][t] = rc.dzg[min(kk, nzg + 1)];
    }
    GeoT<T> gl = g;
    gl.w0 = gys[2] - (j0 - 1);
    gl.w1 = gys[3] - (j0 - 1);
    RcpT<T> rcs;
    rcs.dx = gxs[0] - (i0 - 1);
    rcs.dxg = gxs[1] - (i0 - 1);
    rcs.dy = gys[0] - (j0 - 1);
    rcs.dyg = gys[1] - (j0 - 1);
    rcs.dz = gzs[0] - kb;
    rcs.dzg = gzs[1] - kb;
    const bool du = i <= nx - 1 && j <= nyg - 1, dv = i <= ilim && j <= ny - 1, dw = i <= ilim && j <= nyg - 1;
    // this thread's tile elements (same for every plane and field)
    int eia[NL], eja[NL], erem[NL];
#pragma unroll
    for (int q = 0; q < NL; q++) {
        int rem = threadIdx.x + q * NT;
        erem[q] = rem;
        int sy = rem / SX, sx = rem - sy * SX;
        eia[q] = i0 + sx - 1;
        eja[q] = j0 + sy - 1;
    }
    // nu_t from |S|: per element the plane coefficient (with the ghost-row
    // sign folded in; 0 outside the field) and the (i, j) part of the
    // canonical index are fixed for the whole march
    T ncf[NL], nsg[NL];
    int nbase[NL];
    const long nplane = (long)ns.nxp * ns.nym;
    if (ns.S) {
#pragma unroll
        for (int q = 0; q < NL; q++) {
            const int ia = eia[q], ja = eja[q];
            const bool ok = erem[q] < NP && ia <= nxg && ja <= nyg;
            const int jj = ja == 1 ? 2 : (ja == nyg ? nyg - 1 : ja);
            nsg[q] = ok ? ((jj != ja && ns.dirichlet) ? T(-1) : T(1)) : T(0);
            ncf[q] = ok ? T(-0.5) * ns.C[jj] : T(0);
            nbase[q] = ok ? (wrapn(ia, ns.nxp) - 2) + ns.nxp * (jj - 2) : 0;
        }
    }
    // all loads of one plane are issued before any of them is used; the
    // (i, j) part of every element's index and its in-field mask are fixed
    int oU[NL], oV[NL], oW[NL], oN[NL];
    bool mU[NL], mV[NL], mW[NL], mN[NL];
#pragma unroll
    for (int q = 0; q < NL; q++) {
        const int ia = eia[q], ja = eja[q];
        const bool in = erem[q] < NP;
        mU[q] = in && ia <= nx && ja <= nyg;
        mV[q] = in && ia <= nxg && ja <= ny;
        mW[q] = in && ia <= nxg && ja <= nyg;
        mN[q] = ns.S ? nsg[q] != T(0) : mW[q];
        oU[q] = mU[q] ? U.idx(ia, ja, 0) : 0;
        oV[q] = mV[q] ? V.idx(ia, ja, 0) : 0;
        oW[q] = mW[q] ? W.idx(ia, ja, 0) : 0;
        oN[q] = ns.S ? nbase[q] : (mW[q] ? nt.idx(ia, ja, 0) : 0);
    }
    T pre[4][NL];
    auto fetch = [&](int k) {
        const bool kz = k <= nzg, kw = k <= nz;
        const int koff = ns.S ? (int)(nplane * (wrapn(k, ns.nzp) - 2)) : k * nt.sz;
        const T *Np = ns.S ? ns.S : nt.p;
#pragma unroll
        for (int q = 0; q < NL; q++) {
            pre[0][q] = (mU[q] && kz) ? U.p[oU[q] + k * U.sz] : T(0);
            pre[1][q] = (mV[q] && kz) ? V.p[oV[q] + k * V.sz] : T(0);
            pre[2][q] = (mW[q] && kw) ? W.p[oW[q] + k * W.sz] : T(0);
            pre[3][q] = (mN[q] && kz) ? Np[oN[q] + koff] : T(0);  // |S| (formed at commit) or nu_t
        }
    };
    auto commit = [&](int slot) {
#pragma unroll
        for (int q = 0; q < NL; q++)
            if (erem[q] < NP) {
#pragma unroll
                for (int f = 0; f < 3; f++) ring[slot][f][erem[q]] = pre[f][q];
                T n = pre[3][q];
                if (ns.S) {
                    // max(-C|S|/2, 0), negated on Dirichlet ghost rows (nsg = -1), 0 outside (nsg = 0)
                    const T v = ncf[q] * n;
                    n = nsg[q] * (v > T(0) ? v : T(0));
                }
                ring[slot][3][erem[q]] = n;
            }
    };
    fetch(kb - 1);
    commit(0);
    fetch(kb);
    commit(1);
    fetch(kb + 1);
    commit(2);
    __syncthreads();
    // the z-face fluxes below the chunk's first plane, carried up the march
    T fzu, fzv, fzw;
    {
        RingAcc<T, TX, TY> aU, aV, aW, aN;
        aU.b[0] = ring[0][0]; aU.b[1] = ring[1][0]; aU.b[2] = ring[2][0];
        aV.b[0] = ring[0][1]; aV.b[1] = ring[1][1]; aV.b[2] = ring[2][1];
        aW.b[0] = ring[0][2]; aW.b[1] = ring[1][2]; aW.b[2] = ring[2][2];
        aN.b[0] = ring[0][3]; aN.b[1] = ring[1][3]; aN.b[2] = ring[2][3];
        aU.i0 = aV.i0 = aW.i0 = aN.i0 = i0;
        aU.j0 = aV.j0 = aW.j0 = aN.j0 = j0;
        aU.kc = aV.kc = aW.kc = aN.kc = kb;
        rhs_zflux_dn<T, RingAcc<T, TX, TY>>(gl, rcs, aU, aV, aW, aN, nu, i, j, kb, fzu, fzv, fzw);
    }
    // the ring slots of planes k-1, k, k+1 rotate at run time: one copy of
    // the plane's code (a march unrolled by three, with compile-time slots,
    // triples the code of this large loop body and ran 5 % slower)
    const int bu = out.u.idx(i, j, 0), bv = out.v.idx(i, j, 0), bw = out.w.idx(i, j, 0);
    const int szu = out.u.sz, szv = out.v.sz, szw = out.w.sz;
    int sm1 = 0, s0 = 1, sp1 = 2;
    for (int k = kb; k <= ke; k++) {
        if (k + 1 <= ke) fetch(k + 2);  // in flight during this plane's work
        // RK operands of this plane, loaded before the stencil work; every
        // field of a component has that component's shape
        const bool cu = du && k <= klim, cv = dv && k <= klim, cw = dw && k <= nz - 1;
        const int iu = bu + k * szu, iv = bv + k * szv, iw = bw + k * szw;
        T fu = T(0), fv = T(0), fw = T(0), ou = T(0), ov = T(0), ow = T(0), lu = T(0), lv = T(0), lw = T(0);
        if (cu) { ou = Uo.u.p[iu]; if constexpr (LO) lu = Uolo.u.p[iu]; if constexpr (S > 1) fu = F1.u.p[iu]; }
        if (cv) { ov = Uo.v.p[iv]; if constexpr (LO) lv = Uolo.v.p[iv]; if constexpr (S > 1) fv = F1.v.p[iv]; }
        if (cw) { ow = Uo.w.p[iw]; if constexpr (LO) lw = Uolo.w.p[iw]; if constexpr (S > 1) fw = F1.w.p[iw]; }
        RingAcc<T, TX, TY> aU, aV, aW, aN;
        aU.b[0] = ring[sm1][0]; aU.b[1] = ring[s0][0]; aU.b[2] = ring[sp1][0];
        aV.b[0] = ring[sm1][1]; aV.b[1] = ring[s0][1]; aV.b[2] = ring[sp1][1];
        aW.b[0] = ring[sm1][2]; aW.b[1] = ring[s0][2]; aW.b[2] = ring[sp1][2];
        aN.b[0] = ring[sm1][3]; aN.b[1] = ring[s0][3]; aN.b[2] = ring[sp1][3];
        aU.i0 = aV.i0 = aW.i0 = aN.i0 = i0;
        aU.j0 = aV.j0 = aW.j0 = aN.j0 = j0;
        aU.kc = aV.kc = aW.kc = aN.kc = k;
        // the three right-hand sides first, every thread (the ring holds the
        // tile and its halo, so the reads stay inside it; points outside the
        // field are not stored): with no store between them the shared-memory
        // reads common to u, v and w are issued once
        const T ru = rhs_u_point<T, RingAcc<T, TX, TY>, RcpT<T>, true>(gl, rcs, aU, aV, aW, aN, nu, dPdx, Om, rot, i,
                                                                          j, k, &fzu);
        const T rv = rhs_v_point<T, RingAcc<T, TX, TY>, RcpT<T>, true>(gl, rcs, aU, aV, aW, aN, nu, Om, rot, i, j, k,
                                                                          &fzv);
        const T rw = rhs_w_point<T, RingAcc<T, TX, TY>, RcpT<T>, true>(gl, rcs, aU, aV, aW, aN, nu, dPdz, i, j, k,
                                                                          &fzw);
        if (cu) rk_apply_at<T, S, LO>(ru, fu, ou, lu, iu, out.u.p, F1.u.p, Unlo.u.p, ca, cb, dt);
        if (cv) rk_apply_at<T, S, LO>(rv, fv, ov, lv, iv, out.v.p, F1.v.p, Unlo.v.p, ca, cb, dt);
        if (cw) rk_apply_at<T, S, LO>(rw, fw, ow, lw, iw, out.w.p, F1.w.p, Unlo.w.p, ca, cb, dt);
        __syncthreads();            // plane k-1 no longer read
        if (k + 1 <= ke) commit(sm1);  // plane k+2 into the freed slot
        __syncthreads();
        const int t0 = sm1;
        sm1 = s0;
        s0 = sp1;
        sp1 = t0;
    }
}

template <typename T, int TX, int TY, int S, bool LO>
__global__ void __launch_bounds__(TX *TY, RhsMinB<T>::v) k_rhs3(const __grid_constant__ Rhs3Args<T> a) {
    rhs3_tile<T, TX, TY, S, LO>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One launch over the tiles of several channels (an ensemble): member m owns
// blocks first[m] .. first[m+1]-1, in the order of its own launch's grid.
template <typename T>
struct Rhs3Batch {
    int n;
    int first[CF_ENS_MAXM + 1];
    Rhs3Args<T> a[CF_ENS_MAXM];
};

template <typename T, int TX, int TY, int S, bool LO>
__global__ void __launch_bounds__(TX *TY, RhsMinB<T>::v) k_rhs3_batch(const __grid_constant__ Rhs3Batch<T> B) {
    const int bid = blockIdx.x;
    int m = 0;
    while (m + 1 < B.n && bid >= B.first[m + 1]) m++;
    const int l = bid - B.first[m], ntx = B.a[m].ntx, nty = B.a[m].nty;
    rhs3_tile<T, TX, TY, S, LO>(B.a[m], l % ntx, (l / ntx) % nty, l / (ntx * nty));
}

template <typename T>
static Rhs3Args<T> rhs3_args(cf_ctx *ctx, int s, int src, int dst) {
    constexpr int TX = 32, TY = 8;
    Rhs3Args<T> A;
    GeoT<T> g = geo_of<T>(ctx);
    Fld<T> U = make_fld<T>(ctx->U[src], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[src], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[src], ctx->nxg, ctx->nyg);
    Fld<T> nt = make_fld<T>(ctx->nut, ctx->nxg, ctx->nyg);
    auto trio = [&](void *a, void *b, void *c) {
        Trio<T> t;
        t.u = make_fld<T>(a, ctx->nx, ctx->nyg);
        t.v = make_fld<T>(b, ctx->nxg, ctx->ny);
        t.w = make_fld<T>(c, ctx->nxg, ctx->nyg);
        return t;
    };
    const int o = ctx->old;
    Trio<T> out = trio(ctx->U[dst], ctx->V[dst], ctx->W[dst]);
    Trio<T> F1 = trio(ctx->F[0][0], ctx->F[0][1], ctx->F[0][2]);
    Trio<T> Uo = trio(ctx->U[o], ctx->V[o], ctx->W[o]);
    Trio<T> Uolo = trio(ctx->Ulo[o], ctx->Vlo[o], ctx->Wlo[o]);
    Trio<T> Unlo = s == 3 ? trio(ctx->Ulo[dst], ctx->Vlo[dst], ctx->Wlo[dst]) : trio(nullptr, nullptr, nullptr);
    // canonical cells only (i <= nxp+1, k <= nzp+1): the periodic duplicate
    // column of V, W and plane of U, V are rewritten by the boundary
    // conditions after the projection and read by nothing before them (the
    // divergence takes canonical cells only)
    const int ilim = ctx->nxp + 1, klim = ctx->nzp + 1;
    int ntx = cdiv(ilim - 1, TX), nty = cdiv(ctx->nyg - 2, TY);
    int nkc = std::max(ctx->rhs_nkc > 0 ? ctx->rhs_nkc : 1, cdiv(ctx->nzp, RHS_ZMAX));
    int kc_len = cdiv(klim - 1, nkc);
    const RkCoef rk = rk_coefs();  // F1 and r weights of substep s, rounded to T
    NutSrc<T> ns = {};
    if (ctx->nut_lazy) {
        ns.S = (const T *)ctx->dsm_q + 15 * ctx->nCan;  // |S| slot of the canonical scratch
        ns.C = sizeof(T) == 8 ? (const T *)ctx->avg_nu_t : (const T *)(ctx->avg_nu_t + ctx->nyg + 2);
        ns.nxp = ctx->nxp;
        ns.nym = ctx->nym;
        ns.nzp = ctx->nzp;
        ns.dirichlet = ctx->prm.Dirichlet_nu_t == 1;
    }
    A.g = g;
    A.rc = rcp_of<T>(ctx);
    A.U = U; A.V = V; A.W = W; A.nt = nt;
    A.ns = ns;
    A.ds = ctx->ds;
    A.nu = (T)ctx->prm.nu;
    A.Om = (T)ctx->omega_z;
    A.rot = fabs(ctx->omega_z) > 1e-6 ? 1 : 0;
    A.out = out; A.F1 = F1; A.Uo = Uo; A.Uolo = Uolo; A.Unlo = Unlo;
    A.s = s;
    A.ca = T(s == 1 ? rk.c[1][1] : (s == 2 ? rk.c[2][1] : rk.c[3][1]));
    A.cb = T(s == 1 ? 0.0 : (s == 2 ? rk.c[2][2] : rk.c[3][3]));
    A.kc_len = kc_len;
    A.ilim = ilim;
    A.klim = klim;
    A.ntx = ntx;
    A.nty = nty;
    A.nkc = cdiv(klim - 1, kc_len);
    return A;
}

template <typename T>
int launch_rhs3(cf_ctx *ctx, int s, int src, int dst) {
    constexpr int TX = 32, TY = 8;
    const Rhs3Args<T> A = rhs3_args<T>(ctx, s, src, dst);
    const dim3 grd(A.ntx, A.nty, A.nkc);
    const bool lo = sizeof(T) == 4 && A.Uolo.u.p != nullptr;
#define CF_RHS3(SS, LL) k_rhs3<T, TX, TY, SS, LL><<<grd, TX * TY, 0, ctx->st>>>(A)
    if constexpr (sizeof(T) == 4) {
        if (lo) {
            if (s == 1) CF_RHS3(1, true); else if (s == 2) CF_RHS3(2, true); else CF_RHS3(3, true);
        }
    }
    if (!lo) {
        if (s == 1) CF_RHS3(1, false); else if (s == 2) CF_RHS3(2, false); else CF_RHS3(3, false);
    }
#undef CF_RHS3
    count_launch(ctx, "k_rhs3");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// The fused right-hand sides + RK update of substep s of n channels (state
// buffers src[q] -> dst[q]) in one launch: per channel exactly the
// arithmetic of launch_rhs3.
template <typename T>
int launch_rhs3_batch(cudaStream_t st, cf_ctx *const *m, int s, const int *src, const int *dst, int n) {
    constexpr int TX = 32, TY = 8;
    if (n < 1 || n > CF_ENS_MAXM) return CF_ERR_INVALID;
    Rhs3Batch<T> B;
    B.n = n;
    B.first[0] = 0;
    for (int q = 0; q < n; q++) {
        B.a[q] = rhs3_args<T>(m[q], s, src[q], dst[q]);
        B.first[q + 1] = B.first[q] + B.a[q].ntx * B.a[q].nty * B.a[q].nkc;
    }
    // one variant for all members: the substep is common, the low words
    // must be too
    const bool lo = sizeof(T) == 4 && B.a[0].Uolo.u.p != nullptr;
    for (int q = 1; q < n; q++)
        if ((sizeof(T) == 4 && B.a[q].Uolo.u.p != nullptr) != lo) return CF_ERR_INVALID;
#define CF_RHS3B(SS, LL) k_rhs3_batch<T, TX, TY, SS, LL><<<B.first[n], TX * TY, 0, st>>>(B)
    if constexpr (sizeof(T) == 4) {
        if (lo) {
            if (s == 1) CF_RHS3B(1, true); else if (s == 2) CF_RHS3B(2, true); else CF_RHS3B(3, true);
        }
    }
    if (!lo) {
        if (s == 1) CF_RHS3B(1, false); else if (s == 2) CF_RHS3B(2, false); else CF_RHS3B(3, false);
    }
#undef CF_RHS3B
    return cudaGetLastError() == cudaSuccess ? 0 : CF_ERR_CUDA;
}

// resident fused-RHS blocks per SM (for the z-chunk plan)
int rhs3_blocks_per_sm(int esz) {
    int n = 1;
    if (esz == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_rhs3<float, 32, 8, 2, true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_rhs3<double, 32, 8, 2, false>, 256, 0);
    return n < 1 ? 1 : n;
}

template <typename T>
int launch_rhs(cf_ctx *ctx, int comp, int slot) {
    return rhs_launch<T>(ctx, comp, ctx->cur, 0, 0, slot, 0);
}

template <typename T>
int launch_rhs3(cf_ctx *ctx, int s, int src, int dst);

template <typename T>
int launch_rhs_update(cf_ctx *ctx, int s, int src, int dst) {
    if (ctx->use_rhs3) return launch_rhs3<T>(ctx, s, src, dst);
    for (int c = 0; c < 3; c++) {
        int rc = rhs_launch<T>(ctx, c, src, 1, s, 0, dst);
        if (rc) return rc;
    }
    return 0;
}

// RK update from stored slots (time_integration.f90:108-146), U = Uo + dt*sum
template <typename T>
__global__ void k_rk_update(Fld<T> U, Fld<T> Uo, Fld<T> F1, Fld<T> F2, Fld<T> F3, const DevScal *ds, int s, RkCoef rk,
                            int i1, int j1, int k1) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
    int k = blockIdx.z + 2;
    if (i > i1 || j > j1 || k > k1) return;
    double dt = ds->dt, f;
    if (s == 1) f = dt * rk.c[1][1] * (double)F1(i, j, k);
    else if (s == 2) f = dt * (rk.c[2][1] * (double)F1(i, j, k) + rk.c[2][2] * (double)F2(i, j, k));
    else f = dt * (rk.c[3][1] * (double)F1(i, j, k) + rk.c[3][2] * (double)F2(i, j, k) + rk.c[3][3] * (double)F3(i, j, k));
    U(i, j, k) = (T)((double)Uo(i, j, k) + f);
}

template <typename T>
int launch_rk_update(cf_ctx *ctx, int s) {
    RkCoef rk = rk_coefs();
    for (int comp = 0; comp < 3; comp++) {
        int i1, j1, k1, n1, n2;
        if (comp == 0) { i1 = ctx->nx - 1; j1 = ctx->nyg - 1; k1 = ctx->nzg - 1; n1 = ctx->nx; n2 = ctx->nyg; }
        else if (comp == 1) { i1 = ctx->nxg - 1; j1 = ctx->ny - 1; k1 = ctx->nzg - 1; n1 = ctx->nxg; n2 = ctx->ny; }
        else { i1 = ctx->nxg - 1; j1 = ctx->nyg - 1; k1 = ctx->nz - 1; n1 = ctx->nxg; n2 = ctx->nyg; }
        void **cur = comp == 0 ? ctx->U : comp == 1 ? ctx->V : ctx->W;
        Fld<T> U = make_fld<T>(cur[ctx->cur], n1, n2), Uo = make_fld<T>(cur[ctx->old], n1, n2);
        Fld<T> F1 = make_fld<T>(ctx->F[0][comp], n1, n2), F2 = make_fld<T>(ctx->F[1][comp], n1, n2),
               F3 = make_fld<T>(ctx->F[2][comp], n1, n2);
        dim3 blk(32, 4, 1), grd(cdiv(i1 - 1, 32), cdiv(j1 - 1, 4), k1 - 1);
        k_rk_update<T><<<grd, blk, 0, ctx->st>>>(U, Uo, F1, F2, F3, ctx->ds, s, rk, i1, j1, k1);
        count_launch(ctx, "k_rk_update");
    }
    CF_CUDA(cudaGetLastError());
    return 0;
}

template <typename T>
__global__ void k_copy(const T *a, T *b, long n) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = a[t];
}

template <typename T>
int launch_copy_state(cf_ctx *ctx, int src, int dst) {
    size_t n[3] = {ctx->nU, ctx->nV, ctx->nW};
    void **f[3] = {ctx->U, ctx->V, ctx->W};
    void **lo[3] = {ctx->Ulo, ctx->Vlo, ctx->Wlo};
    for (int c = 0; c < 3; c++) {
        CF_CUDA(cudaMemcpyAsync(f[c][dst], f[c][src], n[c] * sizeof(T), cudaMemcpyDeviceToDevice, ctx->st));
        if (lo[c][src] && lo[c][dst])
            CF_CUDA(cudaMemcpyAsync(lo[c][dst], lo[c][src], n[c] * sizeof(T), cudaMemcpyDeviceToDevice, ctx->st));
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Mass flow, mass_flow.f90.  Block partial sums + a fixed-order final sum so
// the result does not depend on scheduling.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffff, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) r += sh[q];
    __syncthreads();
    return r;
}

// mode 1: trapezoid of U (mass_flow.f90:116-123):
//   sum_{j=3}^{nyg-1} (U_j + U_{j-1}) (yg_j - yg_{j-1})/2 = sum_j c_j sum_i U_ij
// with c_j the two adjacent half-intervals.  Block (k plane, MASS_JR rows),
// one warp per row at a time: the row sum over i is accumulated
// compensated (hi + lo TwoSum) in the state's precision, so that the FP64
// work is one multiply-add per row.
constexpr int MASS_JR = 16;
template <typename T>
__global__ void __launch_bounds__(256) k_mass_partial(Fld<T> U, const double *yg, int nx, int nyg, double *part) {
    __shared__ double sh[8];
    const int k = blockIdx.x + 2, j0 = 2 + blockIdx.y * MASS_JR;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double acc = 0.0;
    for (int r = wp; r < MASS_JR; r += nw) {
        const int j = j0 + r;
        if (j > nyg - 1) break;
        double rsum;
        if constexpr (sizeof(T) == 4) {
            // lanes and the warp tree in float-float: no FP64 per element or per lane
            float hi = 0.f, lo = 0.f;
#pragma unroll 8
            for (int i = lane + 2; i <= nx - 1; i += 32) ff_add(hi, lo, U(i, j, k));
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
                ff_add(hi, lo, oh);
                lo += ol;
            }
            rsum = (double)hi + (double)lo;
        } else {
            rsum = 0.0;
#pragma unroll 8
            for (int i = lane + 2; i <= nx - 1; i += 32) rsum += U(i, j, k);
            for (int o = 16; o > 0; o >>= 1) rsum += __shfl_down_sync(0xffffffffu, rsum, o);
        }
        if (lane == 0) {
            const double c = (j >= 3 ? 0.5 * (yg[j] - yg[j - 1]) : 0.0) + (j <= nyg - 2 ? 0.5 * (yg[j + 1] - yg[j]) : 0.0);
            acc += c * rsum;
        }
    }
    if (lane == 0) sh[wp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < nw; q++) s += sh[q];
        part[blockIdx.x * gridDim.y + blockIdx.y] = s;
    }
}

// mode 1 in the split path, with no FP64 instruction per row or warp (each
// is dozens of times the cost of an FP32 one on this part): the row sum over
// i in float-float, times c_j held as float hi + lo, accumulated per warp and
// per block in float-float; one float-float partial per block.
__global__ void __launch_bounds__(256) k_mass_partial_ff(Fld<float> U, const float2 *cj, int nx, int nyg, float2 *part) {
    __shared__ float2 sh[8];
    const int k = blockIdx.x + 2, j0 = 2 + blockIdx.y * MASS_JR;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float ah = 0.f, al = 0.f;
    for (int r = wp; r < MASS_JR; r += nw) {
        const int j = j0 + r;
        if (j > nyg - 1) break;
        float hi = 0.f, lo = 0.f;
        // the row's loads issued MP at a time before they are summed (a
        // dependent sum per load would wait out the memory latency each time)
        constexpr int MP = 8;
        for (int i0 = lane + 2; i0 <= nx - 1; i0 += 32 * MP) {
            float v[MP];
#pragma unroll
            for (int q = 0; q < MP; q++) v[q] = i0 + 32 * q <= nx - 1 ? U(i0 + 32 * q, j, k) : 0.f;
#pragma unroll
            for (int q = 0; q < MP; q++)
                if (i0 + 32 * q <= nx - 1) ff_add(hi, lo, v[q]);
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
            ff_add(hi, lo, oh);
            lo += ol;
        }
        // lane 0: (hi + lo) * (c.x + c.y), the product's rounding error
        // recovered by an FMA
        const float2 c = cj[j];
        const float p = c.x * hi;
        const float e = fmaf(c.x, hi, -p) + (c.x * lo + c.y * hi);
        ff_add2(ah, al, p, e);
    }
    if (lane == 0) sh[wp] = make_float2(ah, al);
    __syncthreads();
    if (threadIdx.x == 0) {
        float h = 0.f, l = 0.f;
        for (int q = 0; q < nw; q++) ff_add2(h, l, sh[q].x, sh[q].y);
        part[blockIdx.x * gridDim.y + blockIdx.y] = make_float2(h, l);
    }
}

// its final: the float-float partials summed in a fixed order (lane-strided,
// warp tree, block tree), the correction of mode 1 in FP64 by one thread
__global__ void __launch_bounds__(256) k_mass_final_ff(const float2 *part, int n, DevScal *ds, double norm) {
    __shared__ float2 sh[8];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float h = 0.f, l = 0.f;
    for (int q = threadIdx.x; q < n; q += blockDim.x) ff_add2(h, l, part[q].x, part[q].y);
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, h, o), ol = __shfl_down_sync(0xffffffffu, l, o);
        ff_add2(h, l, oh, ol);
    }
    if (lane == 0) sh[wp] = make_float2(h, l);
    __syncthreads();
    if (threadIdx.x != 0) return;
    h = 0.f;
    l = 0.f;
    for (int q = 0; q < nw; q++) ff_add2(h, l, sh[q].x, sh[q].y);
    const double s = (double)h + (double)l;
    ds->mass_sum = s;
    const double corr = ds->Qflow_x_0 - s / norm;
    ds->lmax[2] = corr;  // scratch slot: correction before division by dt
    ds->corrf = (float)corr;
}

// mode 2: centre-line sum (mass_flow.f90:203-204), planes k = 1..nzg-2
template <typename T>
__global__ void k_ucl_partial(Fld<T> U, int nx, int jc, double *part) {
    __shared__ double sh[32];
    int k = blockIdx.x + 1;
    double s = 0.0;
    for (int i = threadIdx.x + 1; i <= nx - 2; i += blockDim.x) s += (double)U(i, jc, k);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// mode 3: trapezoid of V (mass_flow.f90:160-167)
template <typename T>
__global__ void k_massv_partial(Fld<T> V, const double *y, int nxg, int ny, double *part) {
    __shared__ double sh[32];
    int k = blockIdx.x + 2;
    double s = 0.0;
    int ni = nxg - 2, nj = ny - 1;
    for (int t = threadIdx.x; t < ni * nj; t += blockDim.x) {
        int i = t % ni + 2, j = t / ni + 2;
        s += ((double)V(i, j, k) + (double)V(i, j - 1, k)) * 0.5 * (y[j] - y[j - 1]);
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// final: the correction into ds (mass_flow.f90:130, 174, 209); the
// partials are summed in a fixed order (lane-strided, then the block tree)
__global__ void __launch_bounds__(256) k_mass_final(const double *part, int n, DevScal *ds, int mode, double norm) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) s += part[q];
    s = block_sum(s, sh);
    if (threadIdx.x != 0) return;
    ds->mass_sum = s;
    double corr;
    if (mode == 1) corr = ds->Qflow_x_0 - s / norm;
    else if (mode == 2) corr = ds->Ucenterline_x - s / norm;
    else corr = ds->Qflow_y_0 - s / norm;
    ds->lmax[2] = corr;  // scratch slot: correction before division by dt
    ds->corrf = (float)corr;
}

// add the correction to the interior and store dPdx = corr/dt
// (time_integration.f90:154-156, 159-161, 167-169)
// KP planes per thread, every load issued before the first store
constexpr int MASS_KP = 4;
// i0 = 2: interior only (i0..i1, i0..j1, i0..k1).  i0 = 1: the whole array,
// ghosts included, as apply_boundary_conditions would leave it afterwards:
// +c on the rows 2..j1 (periodic copies included) and wsign*c on the wall
// ghost rows 1 and j1+1 (-1: no-slip ghosts of U, 0: the wall faces of V).
template <typename T>
__global__ void __launch_bounds__(128) k_mass_apply(Fld<T> F, Fld<T> Flo, DevScal *ds, int i1, int j1, int k1, int mode,
                                                    int i0, int wsign) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + i0;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + i0;
    const int k0 = blockIdx.z * MASS_KP + i0;
    if (i == i0 && j == i0 && k0 == i0) {
        double corr = ds->lmax[2];
        if (mode == 3) ds->dPdy = corr / ds->dt;
        else {
            ds->dPdx = corr / ds->dt;
            ds->dPdxf = (float)ds->dPdx;
        }
    }
    if (i > i1 || j > j1) return;
    const bool wall = i0 == 1 && (j == 1 || j == j1);
    if (wall && wsign == 0) return;
    T h[MASS_KP], l[MASS_KP];
    const bool lo = Flo.p != nullptr;
#pragma unroll
    for (int q = 0; q < MASS_KP; q++) {
        const int k = k0 + q;
        h[q] = k <= k1 ? F(i, j, k) : T(0);
        l[q] = (lo && k <= k1) ? Flo(i, j, k) : T(0);
    }
    if constexpr (sizeof(T) == 4) {
        const float c = wall ? -ds->corrf : ds->corrf;
#pragma unroll
        for (int q = 0; q < MASS_KP; q++) {
            const int k = k0 + q;
            if (k > k1) break;
            if (lo) {
                float hi = h[q], lw = l[q];
                ff_add(hi, lw, c);
                F(i, j, k) = hi;
                Flo(i, j, k) = lw;
            } else {
                F(i, j, k) = h[q] + c;
            }
        }
    } else {
        const double c = wall ? -ds->lmax[2] : ds->lmax[2];
#pragma unroll
        for (int q = 0; q < MASS_KP; q++)
            if (k0 + q <= k1) F(i, j, k0 + q) = h[q] + c;
    }
}

template <typename T>
static int mass_partial(cf_ctx *ctx, int b, int mode) {
    double *part = ctx->d_red;
    int nb = ctx->nzg - 2;
    double norm;
    if (mode == 1 && sizeof(T) == 4) {
        const int njc = cdiv(ctx->nyg - 2, MASS_JR);
        k_mass_partial_ff<<<dim3(nb, njc), 256, 0, ctx->st>>>(make_fld<float>(ctx->U[b], ctx->nx, ctx->nyg),
                                                               ctx->d_mass_c, ctx->nx, ctx->nyg, (float2 *)part);
        count_launch(ctx, "k_mass_partial");
        k_mass_final_ff<<<1, 256, 0, ctx->st>>>((const float2 *)part, nb * njc, ctx->ds, ctx->mass_norm);
        count_launch(ctx, "k_mass_final");
        CF_CUDA(cudaGetLastError());
        return 0;
    }
    if (mode == 1) {
        const int njc = cdiv(ctx->nyg - 2, MASS_JR);
        k_mass_partial<T><<<dim3(nb, njc), 256, 0, ctx->st>>>(make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg), ctx->geo.yg,
                                                               ctx->nx, ctx->nyg, part);
        nb *= njc;
        norm = ctx->mass_norm;
    } else if (mode == 2) {
        int jc = ctx->ny / 2 + 1;
        k_ucl_partial<T><<<nb, 256, 0, ctx->st>>>(make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg), ctx->nx, jc, part);
        norm = (double)(ctx->nx - 2) * (double)(ctx->nzg - 2);
    } else {
        k_massv_partial<T><<<nb, 256, 0, ctx->st>>>(make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny), ctx->geo.y, ctx->nxg,
                                                     ctx->ny, part);
        norm = ctx->mass_norm_vv;
    }
    count_launch(ctx, "k_mass_partial");
    k_mass_final<<<1, 256, 0, ctx->st>>>(part, nb, ctx->ds, mode, norm);
    count_launch(ctx, "k_mass_final");
    CF_CUDA(cudaGetLastError());
    return 0;
}

template <typename T>
int launch_mass_value(cf_ctx *ctx, int b, int mode) {
    return mass_partial<T>(ctx, b, mode);
}

template <typename T>
int launch_mass_flow(cf_ctx *ctx, int b, int mode, bool ghosts) {
    int rc = mass_partial<T>(ctx, b, mode);
    if (rc) return rc;
    return launch_mass_apply<T>(ctx, b, mode, ghosts);
}

template <typename T>
int launch_mass_apply(cf_ctx *ctx, int b, int mode, bool ghosts) {
    dim3 blk(32, 4, 1);
    if (mode == 3) {
        if (ghosts) {
            int i1 = ctx->nxg, j1 = ctx->ny, k1 = ctx->nzg;
            k_mass_apply<T><<<dim3(cdiv(i1, 32), cdiv(j1, 4), cdiv(k1, MASS_KP)), blk, 0, ctx->st>>>(
                make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny), make_fld<T>(ctx->Vlo[b], ctx->nxg, ctx->ny), ctx->ds, i1, j1,
                k1, mode, 1, 0);
        } else {
            int i1 = ctx->nxg - 1, j1 = ctx->ny - 1, k1 = ctx->nzg - 1;
            k_mass_apply<T><<<dim3(cdiv(i1 - 1, 32), cdiv(j1 - 1, 4), cdiv(k1 - 1, MASS_KP)), blk, 0, ctx->st>>>(
                make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny), make_fld<T>(ctx->Vlo[b], ctx->nxg, ctx->ny), ctx->ds, i1, j1,
                k1, mode, 2, 0);
        }
    } else {
        if (ghosts) {
            int i1 = ctx->nx, j1 = ctx->nyg, k1 = ctx->nzg;
            k_mass_apply<T><<<dim3(cdiv(i1, 32), cdiv(j1, 4), cdiv(k1, MASS_KP)), blk, 0, ctx->st>>>(
                make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg), make_fld<T>(ctx->Ulo[b], ctx->nx, ctx->nyg), ctx->ds, i1, j1,
                k1, mode, 1, -1);
        } else {
            int i1 = ctx->nx - 1, j1 = ctx->nyg - 1, k1 = ctx->nzg - 1;
            k_mass_apply<T><<<dim3(cdiv(i1 - 1, 32), cdiv(j1 - 1, 4), cdiv(k1 - 1, MASS_KP)), blk, 0, ctx->st>>>(
                make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg), make_fld<T>(ctx->Ulo[b], ctx->nx, ctx->nyg), ctx->ds, i1, j1,
                k1, mode, 2, 0);
        }
    }
    count_launch(ctx, "k_mass_apply");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// compute_dt, time_integration.f90:179-227.  max over (i,j,k) of dx_i/|U| is
// dx_i / min_{j,k}|U| exactly (division by a positive number is monotone), so
// the kernel reduces min|U| per x index, min|V| per y index, min|W| per z
// index and a second kernel forms the maxima.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void atomic_min_pos(double *a, double v) {
    // non-negative doubles order like their bit patterns
    atomicMin((unsigned long long *)a, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_pos(double *a, double v) {
    atomicMax((unsigned long long *)a, (unsigned long long)__double_as_longlong(v));
}

// CORR: the corrected convective limit of cf_params.cfl_corrected, which
// needs the maxima of |u| per index instead (same blocks and atomics).  The
// extrema are kept in the state's precision: FP32 ones as the bit patterns of
// non-negative floats (which order like unsigned integers) with 32-bit
// atomics, FP64 ones as 64-bit patterns; widening a float to double is exact,
// so the quotients of the finaliser do not depend on the storage.
template <typename T, bool CORR>
__global__ void __launch_bounds__(256) k_dt_min(Fld<T> U, Fld<T> V, Fld<T> W, int nxg, int nyg, int nzg, T *mu, T *mv,
                                                T *mw) {
    // block (x: up to 256 x indices, y: JR rows, z: KR planes), thread = x index i:
    // min |U| per i over the block's rows
    // and planes, min |V| per row, min |W| per plane; all loads of a plane's
    // rows are issued together.  One global atomic per index per block.
    constexpr int JR = 16, KR = 2;
    __shared__ T vsm[8][JR];
    __shared__ T wsm[8][KR];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int i = 2 + blockIdx.x * blockDim.x + threadIdx.x, j0 = 2 + blockIdx.y * JR, k0 = 2 + blockIdx.z * KR;
    const T init = CORR ? T(0) : T(INFINITY);
    auto ext = [](T a, T b) { return CORR ? fmax(a, b) : fmin(a, b); };
    T umin = init;
    T vmin[JR];
#pragma unroll
    for (int r = 0; r < JR; r++) vmin[r] = init;
#pragma unroll
    for (int kk = 0; kk < KR; kk++) {
        const int k = k0 + kk;
        T wmin = init;
        if (k <= nzg - 1 && i <= nxg - 1) {
            T u[JR], v[JR], w[JR];
#pragma unroll
            for (int r = 0; r < JR; r++) {
                const int j = min(j0 + r, nyg - 1);  // clamped rows repeat row nyg-1
                u[r] = U(i, j, k);
                v[r] = V(i, j, k);
                w[r] = W(i, j, k);
            }
#pragma unroll
            for (int r = 0; r < JR; r++) {
                umin = ext(umin, fabs(u[r]));
                vmin[r] = ext(vmin[r], fabs(v[r]));
                wmin = ext(wmin, fabs(w[r]));
            }
        }
        for (int o = 16; o > 0; o >>= 1) wmin = ext(wmin, __shfl_down_sync(0xffffffff, wmin, o));
        if (lane == 0) wsm[wp][kk] = wmin;
    }
#pragma unroll
    for (int r = 0; r < JR; r++) {
        T v = vmin[r];
        for (int o = 16; o > 0; o >>= 1) v = ext(v, __shfl_down_sync(0xffffffff, v, o));
        if (lane == 0) vsm[wp][r] = v;
    }
    auto put = [](T *a, T v) {
        if constexpr (sizeof(T) == 4) {
            if (CORR) atomicMax((unsigned *)a, __float_as_uint(v));
            else atomicMin((unsigned *)a, __float_as_uint(v));
        } else {
            if (CORR) atomic_max_pos(a, v);
            else atomic_min_pos(a, v);
        }
    };
    if (i <= nxg - 1) put(&mu[i], umin);
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (threadIdx.x < JR) {
        const int j = j0 + threadIdx.x;
        if (j <= nyg - 1) {
            T m = vsm[0][threadIdx.x];
            for (int q = 1; q < nw; q++) m = ext(m, vsm[q][threadIdx.x]);
            put(&mv[j], m);
        }
    } else if (threadIdx.x < JR + KR) {  // JR + KR <= 32: present in a one-warp block too
        const int kk = threadIdx.x - JR, k = k0 + kk;
        if (k <= nzg - 1) {
            T m = wsm[0][kk];
            for (int q = 1; q < nw; q++) m = ext(m, wsm[q][kk]);
            put(&mw[k], m);
        }
    }
}


// The maxima dx/min|u| per direction (one FP64 quotient per thread), dt, and
// the minima reset to +inf for the next call.  corr: the minima dx/max|u|
// instead, the maxima reset to 0.  The quotients are non-negative, so their
// extrema are taken on the 64-bit patterns with integer compares (FP64
// max/min chains are slow on this part); a NaN quotient is skipped like
// fmax/fmin skip it.
template <typename T>
__global__ void __launch_bounds__(1024) k_dt_final(T *mu, T *mv, T *mw, Geo g, DevScal *ds, double CFL, double dt_vis,
                                                   int corr, int advance_t) {
    typedef unsigned long long u64;
    __shared__ u64 sh[3][32];
    const int nxi = g.nxg - 2, nyi = g.nyg - 2, nzi = g.nzg - 2;
    const u64 pinf = 0x7FF0000000000000ull;
    const u64 init = corr ? pinf : 0ull;
    auto ext = [corr](u64 a, u64 b) { return corr ? (a < b ? a : b) : (a > b ? a : b); };
    auto key = [init, pinf](double q) {
        const u64 b = (u64)__double_as_longlong(q);
        return b > pinf ? init : b;
    };
    u64 l[3] = {init, init, init};
    for (int t = threadIdx.x; t < nxi + nyi + nzi; t += blockDim.x) {
        if (t < nxi) {
            const int i = t + 2;
            l[0] = ext(l[0], key((g.xg[i + 1] - g.xg[i]) / (double)mu[i]));
        } else if (t < nxi + nyi) {
            const int j = t - nxi + 2;
            l[1] = ext(l[1], key((g.yg[j + 1] - g.yg[j]) / (double)mv[j]));
        } else {
            const int k = t - nxi - nyi + 2;
            l[2] = ext(l[2], key((g.zg[k + 1] - g.zg[k]) / (double)mw[k]));
        }
    }
#pragma unroll
    for (int d = 0; d < 3; d++)
        for (int o = 16; o > 0; o >>= 1) l[d] = ext(l[d], __shfl_down_sync(0xffffffff, l[d], o));
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sh[0][w] = l[0]; sh[1][w] = l[1]; sh[2][w] = l[2]; }
    __syncthreads();
    const T reset = corr ? T(0) : T(INFINITY);
    for (int t = threadIdx.x; t < g.nxg + 2; t += blockDim.x) mu[t] = reset;
    for (int t = threadIdx.x; t < g.nyg + 2; t += blockDim.x) mv[t] = reset;
    for (int t = threadIdx.x; t < g.nzg + 2; t += blockDim.x) mw[t] = reset;
    if (w != 0) return;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        u64 x = lane < nw ? sh[d][lane] : init;
        for (int o = 16; o > 0; o >>= 1) x = ext(x, __shfl_down_sync(0xffffffff, x, o));
        l[d] = x;
    }
    if (lane != 0) return;
    const double lU = __longlong_as_double((long long)l[0]), lV = __longlong_as_double((long long)l[1]),
                 lW = __longlong_as_double((long long)l[2]);
    double du = CFL * lU, dv = CFL * lV, dw = CFL * lW;
    double dt_conv = fmin(du, fmin(dv, dw));
    double dt = fmin(dt_conv, dt_vis);
    dt = fmin(dt, 5e-3);
    if (CFL < 0) dt = -CFL;
    if (ds->fixed_dt > 0) dt = ds->fixed_dt;
    ds->dt = dt;
    ds->dtf = (float)dt;
    // the step's t = to + rk_t(3) dt, rk_t(3) = 1 (time_integration.f90:146);
    // nothing in the step reads t
    if (advance_t) ds->t = ds->t + dt;
    ds->lmax[0] = lU;
    ds->lmax[1] = lV;
}

template <typename T>
int launch_dt(cf_ctx *ctx, int b, bool advance_t) {
    // extrema start at +inf (0 for the corrected rule): set at context
    // creation and reset by k_dt_final; stored in the state's precision
    T *mu = (T *)ctx->d_dtmin, *mv = mu + ctx->nxg + 2, *mw = mv + ctx->nyg + 2;
    // blocks as wide as the x range (whole warps, at most 256 threads): no
    // idle threads, and more of the small blocks resident at once
    const int bx = std::min(256, 32 * cdiv(ctx->nxg - 2, 32));
    const dim3 grd(cdiv(ctx->nxg - 2, bx), cdiv(ctx->nyg - 2, 16), cdiv(ctx->nzg - 2, 2));
    const Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg), V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny),
                 W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    if (ctx->prm.cfl_corrected) k_dt_min<T, true><<<grd, bx, 0, ctx->st>>>(U, V, W, ctx->nxg, ctx->nyg, ctx->nzg, mu, mv, mw);
    else k_dt_min<T, false><<<grd, bx, 0, ctx->st>>>(U, V, W, ctx->nxg, ctx->nyg, ctx->nzg, mu, mv, mw);
    count_launch(ctx, "k_dt_min");
    double CFL = ctx->prm.CFL;
    double vu = CFL * pow(ctx->dxmin, 2.0) / ctx->prm.nu, vv = CFL * pow(ctx->dymin, 2.0) / ctx->prm.nu,
           vw = CFL * pow(ctx->dzmin, 2.0) / ctx->prm.nu;
    double dt_vis = fmin(vu, fmin(vv, vw));
    k_dt_final<T><<<1, 1024, 0, ctx->st>>>(mu, mv, mw, ctx->geo, ctx->ds, CFL, dt_vis, ctx->prm.cfl_corrected ? 1 : 0,
                                           advance_t ? 1 : 0);
    count_launch(ctx, "k_dt_final");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// check_divergence, projection.f90:234-256 (signed max from 0, and max |div|)
// ---------------------------------------------------------------------------

// A NaN divergence in any cell makes both results NaN (a blown-up field is
// reported as such; fmax alone would drop it).  The NaN is the positive
// quiet one, whose bit pattern orders above +Inf for atomic_max_pos.
__device__ __forceinline__ double nan_max(double a, double b) {
    return (isnan(a) || isnan(b)) ? __longlong_as_double(0x7FF8000000000000LL) : fmax(a, b);
}

template <typename T>
__global__ void k_div(Fld<T> U, Fld<T> V, Fld<T> W, Geo g, double *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
    int k = blockIdx.z + 2;
    double d = 0.0, a = 0.0;
    if (i <= g.nxg - 1 && j <= g.nyg - 1) {
        d = ((double)U(i, j, k) - (double)U(i - 1, j, k)) / (g.x[i] - g.x[i - 1]) +
            ((double)V(i, j, k) - (double)V(i, j - 1, k)) / (g.y[j] - g.y[j - 1]) +
            ((double)W(i, j, k) - (double)W(i, j, k - 1)) / (g.z[k] - g.z[k - 1]);
        a = nan_max(fabs(d), 0.0);
        d = nan_max(d, 0.0);
    }
    for (int o = 16; o > 0; o >>= 1) {
        d = nan_max(d, __shfl_down_sync(0xffffffff, d, o));
        a = nan_max(a, __shfl_down_sync(0xffffffff, a, o));
    }
    if (((threadIdx.x + threadIdx.y * blockDim.x) & 31) == 0) {
        atomic_max_pos(&out[0], d);
        atomic_max_pos(&out[1], a);
    }
}

template <typename T>
int launch_div_check(cf_ctx *ctx, int b, double *d_out) {
    CF_CUDA(cudaMemsetAsync(d_out, 0, 2 * sizeof(double), ctx->st));
    dim3 blk(32, 4, 1), grd(cdiv(ctx->nxg - 2, 32), cdiv(ctx->nyg - 2, 4), ctx->nzg - 2);
    k_div<T><<<grd, blk, 0, ctx->st>>>(make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg), make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny),
                                       make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg), ctx->geo, d_out);
    count_launch(ctx, "k_div");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// True when buffer b satisfies the no-slip ghost identities (one kernel and a
// 4-byte read back); false for the wall model, whose ghosts depend on alpha.
template <typename T>
int check_bc(cf_ctx *ctx, int b, bool *ok) {
    *ok = false;
    if (ctx->prm.iwall_model != 0) return 0;
    BcSet s;
    s.f[0] = bc_field(ctx->U[b], ctx->Ulo[b], ctx->nx, ctx->nyg, ctx->nzg, 0, 1, 0, nullptr);
    s.f[1] = bc_field(ctx->V[b], ctx->Vlo[b], ctx->nxg, ctx->ny, ctx->nzg, 1, 1, 1, nullptr);
    s.f[2] = bc_field(ctx->W[b], ctx->Wlo[b], ctx->nxg, ctx->nyg, ctx->nz, 1, 0, 0, nullptr);
    s.nxp = ctx->nxp;
    s.nzp = ctx->nzp;
    s.dyb = s.dyt = 0.0;
    int *flag = (int *)(ctx->d_red + ctx->red_n - 6);
    CF_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), ctx->st));
    const int tot = s.f[0].n + s.f[1].n + s.f[2].n;
    k_bc_check<T><<<cdiv(tot, 256), 256, 0, ctx->st>>>(s, flag);
    CF_CUDA(cudaGetLastError());
    int h = 1;
    CF_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CF_CUDA(cudaStreamSynchronize(ctx->st));
    *ok = h == 0;
    return 0;
}

#define INST(T)                                                      \
    template int launch_rhs3_batch<T>(cudaStream_t, cf_ctx *const *, int, const int *, const int *, int); \
    template int check_bc<T>(cf_ctx *, int, bool *);                 \
    template int launch_bc<T>(cf_ctx *, int, bool);                  \
    template int launch_rhs<T>(cf_ctx *, int, int);                  \
    template int launch_rhs_update<T>(cf_ctx *, int, int, int);      \
    template int launch_rk_update<T>(cf_ctx *, int);                 \
    template int launch_copy_state<T>(cf_ctx *, int, int);           \
    template int launch_mass_flow<T>(cf_ctx *, int, int, bool);      \
    template int launch_mass_value<T>(cf_ctx *, int, int);           \
    template int launch_mass_apply<T>(cf_ctx *, int, int, bool);     \
    template int launch_dt<T>(cf_ctx *, int, bool);                  \
    template int launch_div_check<T>(cf_ctx *, int, double *);
INST(double)
INST(float)
