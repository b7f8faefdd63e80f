// k_poisson.cu -- pseudo-pressure Poisson solve and projection,
// projection.f90:20-225.
//
// The reference transforms each y-plane with a complex 2-D DFT of the real
// divergence (FFTW, projection.f90:83-87), solves one complex tridiagonal
// system per (kx,kz) mode with LAPACK zgtsv (projection.f90:90-113) and
// transforms back (projection.f90:116-120).  Here the x transform is
// real-to-complex (two real lines packed in one complex FFT), only the
// nxp/2+1 non-redundant x modes are solved, and the z transform is complex.
// The solve restates zgtsv's partial-pivoting elimination; the Dyy matrix is
// real, so real and imaginary parts share every multiplier and pivot choice.
// All FFTs are Stockham autosort transforms in shared memory with radices
// 2, 3, 4 and 5 and twiddles from a table of exp(+-2 pi i e/n).
#include "cf_internal.cuh"

template <typename T> struct C2;
template <> struct C2<double> { typedef double2 t; };
template <> struct C2<float> { typedef float2 t; };

template <typename C> __device__ __forceinline__ C cmk(double a, double b) { C r; r.x = a; r.y = b; return r; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }

struct FftPlan {
    int n, nrad, rad[8];
};

// One line of length n held in smem a (ping) / b (pong); the G threads of a
// group (index tid) cooperate; returns the buffer holding the result.
template <typename C>
__device__ C *fft_smem(C *a, C *b, const FftPlan &pl, const C *tw, int tid, int G) {
    const int n = pl.n;
    int Ns = 1;
    for (int s = 0; s < pl.nrad; s++) {
        const int R = pl.rad[s], nb = n / R, step = n / (Ns * R);
        for (int j = tid; j < nb; j += G) {
            int k = j % Ns;
            C v[5];
#pragma unroll
            for (int r = 0; r < 5; r++)
                if (r < R) {
                    v[r] = a[j + r * nb];
                    if (r > 0 && k > 0) v[r] = cmul(v[r], tw[r * k * step]);
                }
            if (R == 2) {
                C t0 = v[0];
                v[0] = cadd(t0, v[1]);
                v[1] = csub(t0, v[1]);
            } else if (R == 4) {
                C w = tw[n / 4];  // sign*i
                C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
                C s13 = cadd(v[1], v[3]), d13 = cmul(csub(v[1], v[3]), w);
                v[0] = cadd(s02, s13);
                v[2] = csub(s02, s13);
                v[1] = cadd(d02, d13);
                v[3] = csub(d02, d13);
            } else if (R == 3) {
                C w = tw[n / 3];  // (-1/2, sign*sqrt(3)/2)
                C t = cadd(v[1], v[2]), u = csub(v[1], v[2]);
                C m;
                m.x = v[0].x + w.x * t.x;
                m.y = v[0].y + w.x * t.y;
                C iu;  // i*sign*sqrt(3)/2 * u
                iu.x = -w.y * u.y;
                iu.y = w.y * u.x;
                v[0] = cadd(v[0], t);
                v[1] = cadd(m, iu);
                v[2] = csub(m, iu);
            } else {  // R == 5, direct
                C o[5];
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    C acc = v[0];
#pragma unroll
                    for (int r = 1; r < 5; r++) acc = cadd(acc, cmul(v[r], tw[((q * r) % 5) * (n / 5)]));
                    o[q] = acc;
                }
#pragma unroll
                for (int q = 0; q < 5; q++) v[q] = o[q];
            }
            int d = (j / Ns) * Ns * R + k;
#pragma unroll
            for (int r = 0; r < 5; r++)
                if (r < R) b[d + r * Ns] = v[r];
        }
        __syncthreads();
        C *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// ---------------------------------------------------------------------------
// Forward: divergence (projection.f90:45-53) of lines (j, k) and (j, k+1),
// packed as real and imaginary parts, complex FFT along x, split into the
// two half spectra.  spec layout: ((kz*nym + j-2)*nxh + kx).
// Block: LP line pairs x GT threads.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_fwd_x(GeoT<T> g, Fld<T> U, Fld<T> V, Fld<T> W, typename C2<T>::t *spec, FftPlan pl,
                        const typename C2<T>::t *tw, int LP) {
    typedef typename C2<T>::t C;
    extern __shared__ unsigned char smraw[];
    C *sm = (C *)smraw;
    const int n = pl.n, G = blockDim.x / LP;
    const int lp = threadIdx.x / G, tid = threadIdx.x % G;
    long pair = (long)blockIdx.x * LP + lp;
    const int nym = g.nym, nzp = g.nzp;
    long npairs = (long)nym * (nzp / 2);
    bool active = pair < npairs;
    int j = 2, k = 2;
    if (active) {
        j = (int)(pair % nym) + 2;
        k = (int)(pair / nym) * 2 + 2;
    }
    C *a = sm + (long)lp * 2 * n, *b = a + n;
    if (active) {
        for (int i = tid + 2; i <= n + 1; i += G) {
            T d0 = (U(i, j, k) - U(i - 1, j, k)) / (g.x[i] - g.x[i - 1]) +
                   (V(i, j, k) - V(i, j - 1, k)) / (g.y[j] - g.y[j - 1]) +
                   (W(i, j, k) - W(i, j, k - 1)) / (g.z[k] - g.z[k - 1]);
            int k1 = k + 1;
            T d1 = (U(i, j, k1) - U(i - 1, j, k1)) / (g.x[i] - g.x[i - 1]) +
                   (V(i, j, k1) - V(i, j - 1, k1)) / (g.y[j] - g.y[j - 1]) +
                   (W(i, j, k1) - W(i, j, k1 - 1)) / (g.z[k1] - g.z[k1 - 1]);
            C z;
            z.x = d0;
            z.y = d1;
            a[i - 2] = z;
        }
    }
    __syncthreads();
    C *r = fft_smem<C>(a, b, pl, tw, tid, G);
    if (!active) return;
    const int nh = n / 2 + 1;
    C *o0 = spec + ((long)(k - 2) * nym + (j - 2)) * nh;
    C *o1 = spec + ((long)(k - 1) * nym + (j - 2)) * nh;
    for (int q = tid; q < nh; q += G) {
        C Zk = r[q], Zc = cconj(r[(n - q) % n]);
        C A, B;
        A.x = T(0.5) * (Zk.x + Zc.x);
        A.y = T(0.5) * (Zk.y + Zc.y);
        // (Zk - Zc)/(2i) = -i/2 (Zk - Zc)
        B.x = T(0.5) * (Zk.y - Zc.y);
        B.y = -T(0.5) * (Zk.x - Zc.x);
        o0[q] = A;
        o1[q] = B;
    }
}

// ---------------------------------------------------------------------------
// Complex FFT along z for LB consecutive kx of one j.  Block: LB lines.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_fft_z(typename C2<T>::t *spec, FftPlan pl, const typename C2<T>::t *tw, int nym, int nh, int LB) {
    typedef typename C2<T>::t C;
    extern __shared__ unsigned char smraw[];
    C *sm = (C *)smraw;
    const int n = pl.n, G = blockDim.x / LB;
    int ngrp = (nh + LB - 1) / LB;
    int j = blockIdx.x / ngrp, kx0 = (blockIdx.x % ngrp) * LB;
    // load: element (line l, position kz) at sm[l*2n + kz]
    for (int t = threadIdx.x; t < LB * n; t += blockDim.x) {
        int l = t % LB, kz = t / LB;
        C v = cmk<C>(0.0, 0.0);
        if (kx0 + l < nh) v = spec[((long)kz * nym + j) * nh + kx0 + l];
        sm[(long)l * 2 * n + kz] = v;
    }
    __syncthreads();
    const int l = threadIdx.x / G, tid = threadIdx.x % G;
    C *a = sm + (long)l * 2 * n, *b = a + n;
    C *r = fft_smem<C>(a, b, pl, tw, tid, G);
    // r is a or b for every line alike (same number of stages)
    long roff = r - a;
    for (int t = threadIdx.x; t < LB * n; t += blockDim.x) {
        int ll = t % LB, kz = t / LB;
        if (kx0 + ll < nh) spec[((long)kz * nym + j) * nh + kx0 + ll] = sm[(long)ll * 2 * n + roff + kz];
    }
}

// ---------------------------------------------------------------------------
// Tridiagonal solve per (kx, kz) along j (projection.f90:90-113).  The
// matrices D(j) = Dyy(j,j) + kxx + kzz (with D(2)*1.5 for the (0,0) mode)
// never change, so zgtsv's elimination -- pivot choices, multipliers and the
// final U factor -- is done once on the host (tri_factor) and a solve only
// replays its right-hand-side operations: one thread per mode, adjacent
// threads adjacent in kx, factors stored (row, kz, kx) for coalescing.
//   fwd q: no pivot: b[q+1] -= m_q b[q]
//          pivot:    (b[q], b[q+1]) <- (b[q+1], b[q] - m_q b[q+1])
//   back:  b[q] = (b[q] - du_q b[q+1] - dl_q b[q+2]) * rd_q
// ---------------------------------------------------------------------------
struct TriFac {
    const double *m, *rd, *du, *dl;  // [nym][nzp][nh]
    const unsigned char *piv;        // [nym][nzp][nh]
};

template <typename T>
__global__ void __launch_bounds__(64) k_tri(typename C2<T>::t *__restrict__ spec, TriFac f, int nym, int nh, int nzp) {
    // 64 modes (consecutive kx, one kz) per block; rows move through shared
    // memory RB at a time with coalesced loads, so each thread's serial
    // recurrence never waits on a global load.
    typedef typename C2<T>::t C;
    constexpr int RB = 16, NT = 64;
    __shared__ C sb[RB][NT];
    __shared__ double sm_[RB][NT], s2[RB][NT], s3[RB][NT];
    __shared__ unsigned char sp[RB][NT];
    const int kx0 = blockIdx.x * NT, kz = blockIdx.y, t = threadIdx.x, kx = kx0 + t;
    const bool act = kx < nh;
    const long stride = nh, fs = (long)nzp * nh, f0 = (long)kz * nh;
    C *col = spec + (long)kz * nym * nh;
    double br = 0.0, bi = 0.0;
    if (act) { C b0 = col[kx]; br = b0.x; bi = b0.y; }
    // forward: rows q = 0 .. nym-2 eliminate into row q+1
    for (int q0 = 0; q0 < nym - 1; q0 += RB) {
        int nr = min(RB, nym - 1 - q0);
        __syncthreads();
        for (int r = 0; r < nr; r++) {
            long off = (long)(q0 + r) * fs + f0 + kx;
            if (act) {
                sb[r][t] = col[(q0 + r + 1) * stride + kx];
                sm_[r][t] = f.m[off];
                sp[r][t] = f.piv[off];
            }
        }
        __syncthreads();
        if (act) {
            for (int r = 0; r < nr; r++) {
                C bn = sb[r][t];
                double nre = bn.x, nim = bn.y, m = sm_[r][t];
                C done;
                if (sp[r][t]) {
                    done = cmk<C>(nre, nim);
                    nre = br - m * nre;
                    nim = bi - m * nim;
                } else {
                    done = cmk<C>(br, bi);
                    nre = nre - m * br;
                    nim = nim - m * bi;
                }
                sb[r][t] = done;  // final row q0 + r
                br = nre;
                bi = nim;
            }
        }
        __syncthreads();
        for (int r = 0; r < nr; r++)
            if (act) col[(q0 + r) * stride + kx] = sb[r][t];
    }
    // back substitution, rows nym-1 .. 0
    double x1r = 0.0, x1i = 0.0, x2r = 0.0, x2i = 0.0;
    if (act) {
        double rd = f.rd[(long)(nym - 1) * fs + f0 + kx];
        x1r = br * rd;
        x1i = bi * rd;
        col[(nym - 1) * stride + kx] = cmk<C>(x1r, x1i);
    }
    for (int q1 = nym - 2; q1 >= 0; q1 -= RB) {
        int nr = min(RB, q1 + 1);
        __syncthreads();
        for (int r = 0; r < nr; r++) {
            int q = q1 - r;
            long off = (long)q * fs + f0 + kx;
            if (act) {
                sb[r][t] = col[q * stride + kx];
                sm_[r][t] = f.rd[off];
                s2[r][t] = f.du[off];
                s3[r][t] = f.dl[off];
            }
        }
        __syncthreads();
        if (act) {
            for (int r = 0; r < nr; r++) {
                C bb = sb[r][t];
                double du = s2[r][t], dl = s3[r][t], rd = sm_[r][t];
                double yr = ((double)bb.x - du * x1r - dl * x2r) * rd;
                double yi = ((double)bb.y - du * x1i - dl * x2i) * rd;
                sb[r][t] = cmk<C>(yr, yi);
                x2r = x1r; x2i = x1i;
                x1r = yr; x1i = yi;
            }
        }
        __syncthreads();
        for (int r = 0; r < nr; r++)
            if (act) col[(q1 - r) * stride + kx] = sb[r][t];
    }
}

// ---------------------------------------------------------------------------
// Inverse x: two half spectra -> one complex sequence -> FFT (+) -> real
// lines (j,k), (j,k+1) into phi (canonical), scaled by 1/(nxp*nzp)
// (projection.f90:116-120).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_inv_x(const typename C2<T>::t *spec, T *phi, FftPlan pl, const typename C2<T>::t *tw, int nym, int nzp,
                        int LP, double scale) {
    typedef typename C2<T>::t C;
    extern __shared__ unsigned char smraw[];
    C *sm = (C *)smraw;
    const int n = pl.n, G = blockDim.x / LP, nh = n / 2 + 1;
    const int lp = threadIdx.x / G, tid = threadIdx.x % G;
    long pair = (long)blockIdx.x * LP + lp;
    long npairs = (long)nym * (nzp / 2);
    bool active = pair < npairs;
    int jj = 0, kk = 0;
    if (active) {
        jj = (int)(pair % nym);
        kk = (int)(pair / nym) * 2;
    }
    C *a = sm + (long)lp * 2 * n, *b = a + n;
    if (active) {
        const C *s0 = spec + ((long)kk * nym + jj) * nh, *s1 = spec + ((long)(kk + 1) * nym + jj) * nh;
        for (int q = tid; q < n; q += G) {
            C A, B;
            if (q < nh) {
                A = s0[q];
                B = s1[q];
                if (q == 0 || 2 * q == n) { A.y = 0; B.y = 0; }
            } else {
                A = cconj(s0[n - q]);
                B = cconj(s1[n - q]);
            }
            C z;  // A + i B
            z.x = A.x - B.y;
            z.y = A.y + B.x;
            a[q] = z;
        }
    }
    __syncthreads();
    C *r = fft_smem<C>(a, b, pl, tw, tid, G);
    if (!active) return;
    long base0 = (long)n * (jj + (long)nym * kk), base1 = (long)n * (jj + (long)nym * (kk + 1));
    for (int q = tid; q < n; q += G) {
        phi[base0 + q] = r[q].x * T(scale);
        phi[base1 + q] = r[q].y * T(scale);
    }
}

// ---------------------------------------------------------------------------
// project_velocity (projection.f90:203-225) and the pressure store of
// rk_step 1 (projection.f90:129-137).  phi is read through the periodic wrap,
// which reproduces apply_periodic_xz_pressure (projection.f90:144-162).
// ---------------------------------------------------------------------------
// valid for i in [2-np, 2np+1]
__device__ __forceinline__ int wrapf(int i, int np) { return i < 2 ? i + np : (i > np + 1 ? i - np : i); }

struct PhiView {
    int nxp, nym, nzp;
    __device__ __forceinline__ long operator()(int i, int j, int k) const {
        return (long)(wrapf(i, nxp) - 2) + (long)nxp * ((j - 2) + (long)nym * (wrapf(k, nzp) - 2));
    }
};

template <typename T, int COMP>
__global__ void k_project(GeoT<T> g, Fld<T> F, Fld<T> Flo, const T *phi, PhiView pv, int i1, int j1, int k1) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
    int k = blockIdx.z + 2;
    if (i > i1 || j > j1 || k > k1) return;
    T grad;
    if (COMP == 0) grad = (phi[pv(i + 1, j, k)] - phi[pv(i, j, k)]) / (g.xg[i + 1] - g.xg[i]);
    else if (COMP == 1) grad = (phi[pv(i, j + 1, k)] - phi[pv(i, j, k)]) / (g.yg[j + 1] - g.yg[j]);
    else grad = (phi[pv(i, j, k + 1)] - phi[pv(i, j, k)]) / (g.zg[k + 1] - g.zg[k]);
    if constexpr (sizeof(T) == 4) {
        if (Flo.p) {
            float hi = F(i, j, k), lo = Flo(i, j, k);
            ff_add(hi, lo, -grad);
            F(i, j, k) = hi;
            Flo(i, j, k) = lo;
            return;
        }
    }
    F(i, j, k) = F(i, j, k) - grad;
}

template <typename T>
__global__ void k_store_p(Fld<T> P, const T *phi, PhiView pv, const DevScal *ds, double c11, int nxg, int nyg, int nzg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int k = blockIdx.z + 1;
    if (i > nxg || j > nyg) return;
    int ic = min(max(i, 2), nxg - 1), jc = min(max(j, 2), nyg - 1), kc = min(max(k, 2), nzg - 1);
    P(i, j, k) = phi[pv(ic, jc, kc)] / (ds_dt<T>(ds) * T(c11));
}

template <typename T>
static size_t smem_pairs(int n, int LP) {
    return (size_t)LP * 2 * n * sizeof(typename C2<T>::t);
}

template <typename T>
int launch_projection(cf_ctx *ctx, int b, bool store_p) {
    typedef typename C2<T>::t C;
    GeoT<T> g = geo_of<T>(ctx);
    Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    C *spec = (C *)ctx->spec;
    T *phi = (T *)ctx->phi;
    const int nxp = ctx->nxp, nzp = ctx->nzp, nym = ctx->nym, nh = ctx->nxh;
    FftPlan px, pz;
    px.n = nxp; px.nrad = ctx->nradx;
    pz.n = nzp; pz.nrad = ctx->nradz;
    for (int q = 0; q < 8; q++) { px.rad[q] = ctx->radx[q]; pz.rad[q] = ctx->radz[q]; }
    // twiddle tables (complex of T): x fwd, x bwd, z fwd, z bwd
    const C *tw = (const C *)ctx->d_tw;
    const C *twxf = tw, *twxb = tw + nxp, *twzf = tw + 2 * nxp, *twzb = tw + 2 * nxp + nzp;
    int minrx = 5, minrz = 5;
    for (int q = 0; q < px.nrad; q++) minrx = min(minrx, px.rad[q]);
    for (int q = 0; q < pz.nrad; q++) minrz = min(minrz, pz.rad[q]);
    int Gx = max(32, ((nxp / minrx + 31) / 32) * 32), Gz = max(32, ((nzp / minrz + 31) / 32) * 32);
    int LP = max(1, 256 / Gx);
    while (LP > 1 && smem_pairs<T>(nxp, LP) > 96 * 1024) LP--;
    long npairs = (long)nym * (nzp / 2);
    size_t shx = smem_pairs<T>(nxp, LP);
    // forward x (divergence fused)
    k_fwd_x<T><<<cdiv(npairs, LP), LP * Gx, shx, ctx->st>>>(g, U, V, W, spec, px, twxf, LP);
    count_launch(ctx, "k_fwd_x");
    // forward z
    int LB = max(1, 256 / Gz);
    while (LB > 1 && smem_pairs<T>(nzp, LB) > 96 * 1024) LB--;
    int ngrp = (nh + LB - 1) / LB;
    size_t shz = smem_pairs<T>(nzp, LB);
    k_fft_z<T><<<nym * ngrp, LB * Gz, shz, ctx->st>>>(spec, pz, twzf, nym, nh, LB);
    count_launch(ctx, "k_fft_z");
    // tridiagonal
    dim3 gt(cdiv(nh, 64), nzp);
    TriFac tf;
    size_t nf = (size_t)nym * nzp * nh;
    tf.m = ctx->tri_fac;
    tf.rd = ctx->tri_fac + nf;
    tf.du = ctx->tri_fac + 2 * nf;
    tf.dl = ctx->tri_fac + 3 * nf;
    tf.piv = ctx->tri_piv;
    k_tri<T><<<gt, 64, 0, ctx->st>>>(spec, tf, nym, nh, nzp);
    count_launch(ctx, "k_tri");
    // inverse z
    k_fft_z<T><<<nym * ngrp, LB * Gz, shz, ctx->st>>>(spec, pz, twzb, nym, nh, LB);
    count_launch(ctx, "k_fft_z");
    // inverse x
    double scale = 1.0 / ((double)nxp * (double)nzp);
    k_inv_x<T><<<cdiv(npairs, LP), LP * Gx, shx, ctx->st>>>(spec, phi, px, twxb, nym, nzp, LP, scale);
    count_launch(ctx, "k_inv_x");
    // projection
    PhiView pv;
    pv.nxp = nxp; pv.nym = nym; pv.nzp = nzp;
    dim3 blk(32, 4, 1);
    {
        int i1 = ctx->nx - 1, j1 = ctx->nyg - 1, k1 = ctx->nzg - 1;
        k_project<T, 0><<<dim3(cdiv(i1 - 1, 32), cdiv(j1 - 1, 4), k1 - 1), blk, 0, ctx->st>>>(
            g, U, make_fld<T>(ctx->Ulo[b], ctx->nx, ctx->nyg), phi, pv, i1, j1, k1);
    }
    {
        int i1 = ctx->nxg - 1, j1 = ctx->ny - 1, k1 = ctx->nzg - 1;
        k_project<T, 1><<<dim3(cdiv(i1 - 1, 32), cdiv(j1 - 1, 4), k1 - 1), blk, 0, ctx->st>>>(
            g, V, make_fld<T>(ctx->Vlo[b], ctx->nxg, ctx->ny), phi, pv, i1, j1, k1);
    }
    {
        int i1 = ctx->nxg - 1, j1 = ctx->nyg - 1, k1 = ctx->nz - 1;
        k_project<T, 2><<<dim3(cdiv(i1 - 1, 32), cdiv(j1 - 1, 4), k1 - 1), blk, 0, ctx->st>>>(
            g, W, make_fld<T>(ctx->Wlo[b], ctx->nxg, ctx->nyg), phi, pv, i1, j1, k1);
    }
    count_launch(ctx, "k_project"); count_launch(ctx, "k_project"); count_launch(ctx, "k_project");
    if (store_p) {
        Fld<T> P = make_fld<T>(ctx->P, ctx->nxg, ctx->nyg);
        k_store_p<T><<<dim3(cdiv(ctx->nxg, 32), cdiv(ctx->nyg, 4), ctx->nzg), blk, 0, ctx->st>>>(
            P, phi, pv, ctx->ds, 8.0 / 15.0, ctx->nxg, ctx->nyg, ctx->nzg);
        count_launch(ctx, "k_store_p");
    }
    CF_CUDA(cudaGetLastError());
    return 0;
}

// smem opt-in for the FFT kernels (called once at context creation)
int fft_setup_attrs() {
    cudaFuncSetAttribute(k_fwd_x<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_fwd_x<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_inv_x<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_inv_x<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_fft_z<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_fft_z<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    return 0;
}

template int launch_projection<double>(cf_ctx *, int, bool);
template int launch_projection<float>(cf_ctx *, int, bool);
