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
#include <algorithm>

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
// The same Stockham transform for a length N known at compile time (the
// common grid sizes): radices, strides and loop bounds are constants, the
// radix sequence is the host plan's (4s, then 2, 3, 5), and the twiddle
// table sits in shared memory.
// ---------------------------------------------------------------------------
constexpr int fft_nrad(int n) {
    int c = 0;
    while (n % 4 == 0) { n /= 4; c++; }
    while (n % 2 == 0) { n /= 2; c++; }
    while (n % 3 == 0) { n /= 3; c++; }
    while (n % 5 == 0) { n /= 5; c++; }
    return n == 1 ? c : -1;
}
constexpr int fft_rad(int n, int s) {
    int c = 0;
    while (n % 4 == 0) { if (c++ == s) return 4; n /= 4; }
    while (n % 2 == 0) { if (c++ == s) return 2; n /= 2; }
    while (n % 3 == 0) { if (c++ == s) return 3; n /= 3; }
    while (n % 5 == 0) { if (c++ == s) return 5; n /= 5; }
    return 1;
}

template <int R, int N, typename C>
__device__ __forceinline__ void butterfly(C *v, const C *tw) {
    if constexpr (R == 2) {
        C t0 = v[0];
        v[0] = cadd(t0, v[1]);
        v[1] = csub(t0, v[1]);
    } else if constexpr (R == 4) {
        const C w = tw[N / 4];  // sign*i
        C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        C s13 = cadd(v[1], v[3]), d13 = cmul(csub(v[1], v[3]), w);
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = cadd(d02, d13);
        v[3] = csub(d02, d13);
    } else if constexpr (R == 3) {
        const C w = tw[N / 3];  // (-1/2, sign*sqrt(3)/2)
        C t = cadd(v[1], v[2]), u = csub(v[1], v[2]);
        C m;
        m.x = v[0].x + w.x * t.x;
        m.y = v[0].y + w.x * t.y;
        C iu;
        iu.x = -w.y * u.y;
        iu.y = w.y * u.x;
        v[0] = cadd(v[0], t);
        v[1] = cadd(m, iu);
        v[2] = csub(m, iu);
    } else {
        static_assert(R == 5, "radix");
        C o[5];
#pragma unroll
        for (int q = 0; q < 5; q++) {
            C acc = v[0];
#pragma unroll
            for (int r = 1; r < 5; r++) acc = cadd(acc, cmul(v[r], tw[((q * r) % 5) * (N / 5)]));
            o[q] = acc;
        }
#pragma unroll
        for (int q = 0; q < 5; q++) v[q] = o[q];
    }
}

template <int N, int S, int NS, typename C>
__device__ __forceinline__ C *fft_fixed(C *a, C *b, const C *tw, int tid, int G) {
    if constexpr (S == fft_nrad(N)) {
        return a;
    } else {
        constexpr int R = fft_rad(N, S), nb = N / R, step = N / (NS * R);
        for (int j = tid; j < nb; j += G) {
            const int k = j % NS;
            C v[R];
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = a[j + r * nb];
            if constexpr (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; r++) v[r] = cmul(v[r], tw[r * k * step]);
            }
            butterfly<R, N>(v, tw);
            const int d = (j / NS) * NS * R + k;
#pragma unroll
            for (int r = 0; r < R; r++) b[d + r * NS] = v[r];
        }
        __syncthreads();
        return fft_fixed<N, S + 1, NS * R, C>(b, a, tw, tid, G);
    }
}

// One line: the compile-time transform when N > 0, else the plan's.
template <int N, typename C>
__device__ __forceinline__ C *fft_line(C *a, C *b, const FftPlan &pl, const C *tw, int tid, int G) {
    if constexpr (N > 0) return fft_fixed<N, 0, 1, C>(a, b, tw, tid, G);
    else return fft_smem<C>(a, b, pl, tw, tid, G);
}

// Copies the twiddle table to shared memory (compile-time sizes only).
template <int N, typename C>
__device__ __forceinline__ const C *stage_twiddles(const C *tw, C *sm_tw) {
    if constexpr (N > 0) {
        for (int e = threadIdx.x; e < N; e += blockDim.x) sm_tw[e] = tw[e];
        return sm_tw;
    } else {
        return tw;
    }
}

// threads per line of the x transforms (the host launch uses the same rule)
__host__ __device__ constexpr int fft_x_threads(int n) { return n >= 128 ? 32 : 16; }

// reciprocal face spacings 1/(x(i)-x(i-1)) etc., 1-based (split path)
struct RSp {
    const float *rx, *ry, *rz;
};

// ---------------------------------------------------------------------------
// Forward: divergence (projection.f90:45-53) of lines (j, k) and (j, k+1),
// packed as real and imaginary parts, complex FFT along x, split into the
// two half spectra.  spec layout: ((kz*nym + j-2)*nxh + kx).
// Block: LP line pairs x GT threads.
// ---------------------------------------------------------------------------
template <typename T, int N>
__global__ void k_fwd_x(GeoT<T> g, Fld<T> U, Fld<T> V, Fld<T> W, typename C2<T>::t *spec, FftPlan pl,
                        const typename C2<T>::t *tw_g, int LP, RSp rs) {
    typedef typename C2<T>::t C;
    extern __shared__ unsigned char smraw[];
    C *sm = (C *)smraw;
    const int n = N > 0 ? N : pl.n, G = N > 0 ? fft_x_threads(N) : blockDim.x / LP;
    const C *tw = stage_twiddles<N, C>(tw_g, sm + (long)LP * 2 * n);
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
    // the x and z neighbours below the first interior index are read through
    // the periodic wrap (U(1) = U(nxp+1), W(k=1) = W(nzp+1)), so the ghosts
    // need not be filled before this kernel
    const int km = k == 2 ? nzp + 1 : k - 1;
    if (active) {
        if constexpr (sizeof(T) == 4 && N > 0) {
            // split path, compile-time length: reciprocal spacings instead of
            // divisions; the loads of XB points are issued before any of them
            // is used or stored (a shared-memory store would otherwise order
            // every later load of U, V, W behind it)
            constexpr int GX = fft_x_threads(N), NPT = N / GX, XB = NPT < 3 ? NPT : 3;
            const float ry = rs.ry[j], rz0 = rs.rz[k], rz1 = rs.rz[k + 1];
            const int k1 = k + 1;
#pragma unroll
            for (int e0 = 0; e0 < NPT; e0 += XB) {
                float ua[XB], uam[XB], ub[XB], ubm[XB], va[XB], vam[XB], vb[XB], vbm[XB], wa[XB], wb[XB], wm[XB], rx[XB];
#pragma unroll
                for (int b = 0; b < XB; b++) {
                    const int i = tid + 2 + (e0 + b) * GX, im = i == 2 ? n + 1 : i - 1;
                    if (e0 + b < NPT) {
                        rx[b] = rs.rx[i];
                        ua[b] = U(i, j, k); uam[b] = U(im, j, k); ub[b] = U(i, j, k1); ubm[b] = U(im, j, k1);
                        va[b] = V(i, j, k); vam[b] = V(i, j - 1, k); vb[b] = V(i, j, k1); vbm[b] = V(i, j - 1, k1);
                        wa[b] = W(i, j, k); wb[b] = W(i, j, k1); wm[b] = W(i, j, km);
                    }
                }
#pragma unroll
                for (int b = 0; b < XB; b++) {
                    if (e0 + b < NPT) {
                        const int i = tid + 2 + (e0 + b) * GX;
                        C z;
                        z.x = (ua[b] - uam[b]) * rx[b] + (va[b] - vam[b]) * ry + (wa[b] - wm[b]) * rz0;
                        z.y = (ub[b] - ubm[b]) * rx[b] + (vb[b] - vbm[b]) * ry + (wb[b] - wa[b]) * rz1;
                        a[i - 2] = z;
                    }
                }
            }
        } else if constexpr (sizeof(T) == 4) {
            // split path, run-time length
            const float ry = rs.ry[j], rz0 = rs.rz[k], rz1 = rs.rz[k + 1];
            for (int i = tid + 2; i <= n + 1; i += G) {
                const float rx = rs.rx[i];
                const int k1 = k + 1, im = i == 2 ? n + 1 : i - 1;
                const float w0 = W(i, j, k), w1 = W(i, j, k1);
                T d0 = (U(i, j, k) - U(im, j, k)) * rx + (V(i, j, k) - V(i, j - 1, k)) * ry +
                       (w0 - W(i, j, km)) * rz0;
                T d1 = (U(i, j, k1) - U(im, j, k1)) * rx + (V(i, j, k1) - V(i, j - 1, k1)) * ry +
                       (w1 - w0) * rz1;
                C z;
                z.x = d0;
                z.y = d1;
                a[i - 2] = z;
            }
        } else {
            for (int i = tid + 2; i <= n + 1; i += G) {
                const int im = i == 2 ? n + 1 : i - 1;
                T d0 = (U(i, j, k) - U(im, j, k)) / (g.x[i] - g.x[i - 1]) +
                       (V(i, j, k) - V(i, j - 1, k)) / (g.y[j] - g.y[j - 1]) +
                       (W(i, j, k) - W(i, j, km)) / (g.z[k] - g.z[k - 1]);
                int k1 = k + 1;
                T d1 = (U(i, j, k1) - U(im, j, k1)) / (g.x[i] - g.x[i - 1]) +
                       (V(i, j, k1) - V(i, j - 1, k1)) / (g.y[j] - g.y[j - 1]) +
                       (W(i, j, k1) - W(i, j, k1 - 1)) / (g.z[k1] - g.z[k1 - 1]);
                C z;
                z.x = d0;
                z.y = d1;
                a[i - 2] = z;
            }
        }
    }
    __syncthreads();
    C *r = fft_line<N, C>(a, b, pl, tw, tid, G);
    if (!active) return;
    const int nh = n / 2 + 1;
    C *o0 = spec + ((long)(j - 2) * nzp + (k - 2)) * nh;
    C *o1 = spec + ((long)(j - 2) * nzp + (k - 1)) * nh;
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
// Complex FFT along z of LB consecutive lines (j, kx), line index j*nh + kx.
// Element kz of a line sits at ((j*nzp + kz)*nh + kx), so for one kz the
// lines of a block are (mostly) adjacent in memory.
// ---------------------------------------------------------------------------
// compile-time z transforms run with 16 lines x 16 threads per block, so a
// thread copies every 16th element of its line
constexpr int FFTZ_KZS = 16;

template <typename T, int N>
__global__ void k_fft_z(typename C2<T>::t *spec, FftPlan pl, const typename C2<T>::t *tw_g, int nlines, int nh, int LB) {
    typedef typename C2<T>::t C;
    extern __shared__ unsigned char smraw[];
    C *sm = (C *)smraw;
    const int n = N > 0 ? N : pl.n, G = blockDim.x / LB;
    const int LS = 2 * n + 1;  // line stride: odd, so that adjacent lines fall in different banks
    const C *tw = stage_twiddles<N, C>(tw_g, sm + (long)LB * LS);
    // blockDim.x is a multiple of LB: a thread keeps one line in the copies
    const int cl = threadIdx.x % LB, kz0 = threadIdx.x / LB, kzs = blockDim.x / LB;
    const long L = (long)blockIdx.x * LB + cl;
    const bool lact = L < nlines;
    long gbase = 0;
    if (lact) {
        const long j = L / nh, kx = L - j * nh;
        gbase = j * n * nh + kx;
    }
    // load: element (line l, position kz) at sm[l*LS + kz]; with a
    // compile-time length every load of the thread is issued first
    if constexpr (N > 0) {
        constexpr int NPT = N / FFTZ_KZS;
        C v[NPT];
#pragma unroll
        for (int e = 0; e < NPT; e++) v[e] = lact ? spec[gbase + (long)(kz0 + e * FFTZ_KZS) * nh] : cmk<C>(0.0, 0.0);
#pragma unroll
        for (int e = 0; e < NPT; e++) sm[(long)cl * LS + kz0 + e * FFTZ_KZS] = v[e];
    } else {
        for (int kz = kz0; kz < n; kz += kzs) sm[(long)cl * LS + kz] = lact ? spec[gbase + (long)kz * nh] : cmk<C>(0.0, 0.0);
    }
    __syncthreads();
    const int l = threadIdx.x / G, tid = threadIdx.x % G;
    C *a = sm + (long)l * LS, *b = a + n;
    C *r = fft_line<N, C>(a, b, pl, tw, tid, G);
    // r is a or b for every line alike (same number of stages)
    long roff = r - a;
    if (lact)
        for (int kz = kz0; kz < n; kz += kzs) spec[gbase + (long)kz * nh] = sm[(long)cl * LS + roff + kz];
}

// ---------------------------------------------------------------------------
// z transforms of the compile-time lengths up to 256 as at most two Stockham
// stages of composite radix (16 = 4x4, 12 = 4x3, 8 = 4x2), each radix-R
// butterfly a register DFT: the first stage reads its R elements straight
// from the spectrum and stores to shared memory, the second reads them back
// and stores its results straight to the spectrum -- one shared-memory round
// trip per element instead of one per radix-2..5 stage plus the copies in
// and out.  Same Stockham ordering as fft_fixed (natural order in and out).
// ---------------------------------------------------------------------------
constexpr int zr_r0(int n) {
    return n == 16 ? 16 : n == 32 ? 8 : n == 64 ? 8 : n == 96 ? 8 : n == 128 ? 16 : n == 192 ? 16 : n == 256 ? 16 : 0;
}
constexpr int zr_r1(int n) {
    return n == 16 ? 1 : n == 32 ? 4 : n == 64 ? 8 : n == 96 ? 12 : n == 128 ? 8 : n == 192 ? 12 : n == 256 ? 16 : 0;
}
// threads per line: the butterflies of both stages spread evenly where the
// counts allow it
constexpr int zr_threads(int n) {
    return n == 16 ? 1 : n == 32 ? 4 : n == 64 ? 8 : n == 96 ? 4 : n == 128 ? 8 : n == 192 ? 16 : n == 256 ? 16 : 0;
}
constexpr int ZR_T = 256;  // threads per block

// DFT of R values in registers (natural order in and out): R = Ra Rb split
// as X[qa + Ra qb] = sum_rb W_Rb^(rb qb) W_R^(rb qa) sum_ra v[Rb ra + rb] W_Ra^(ra qa),
// roots W_R^m = tw[(N/R) m] from the length-N table.
template <int R> constexpr int reg_ra() { return R % 4 == 0 ? 4 : (R % 2 == 0 ? 2 : (R % 3 == 0 ? 3 : 5)); }

template <int R, int N, typename C>
__device__ __forceinline__ void reg_dft(C *v, const C *tw) {
    if constexpr (R == 2 || R == 3 || R == 4 || R == 5) {
        butterfly<R, N>(v, tw);
    } else if constexpr (R > 5) {
        constexpr int Ra = reg_ra<R>(), Rb = R / Ra;
        C u[R];
#pragma unroll
        for (int rb = 0; rb < Rb; rb++) {
            C s[Ra];
#pragma unroll
            for (int ra = 0; ra < Ra; ra++) s[ra] = v[Rb * ra + rb];
            reg_dft<Ra, N>(s, tw);
#pragma unroll
            for (int qa = 0; qa < Ra; qa++) u[rb * Ra + qa] = (rb * qa) ? cmul(s[qa], tw[(N / R) * rb * qa]) : s[qa];
        }
#pragma unroll
        for (int qa = 0; qa < Ra; qa++) {
            C s[Rb];
#pragma unroll
            for (int rb = 0; rb < Rb; rb++) s[rb] = u[rb * Ra + qa];
            reg_dft<Rb, N>(s, tw);
#pragma unroll
            for (int qb = 0; qb < Rb; qb++) v[qa + Ra * qb] = s[qb];
        }
    }
}

template <typename T, int N>
__global__ void __launch_bounds__(ZR_T) k_fft_zr(typename C2<T>::t *__restrict__ spec,
                                                 const typename C2<T>::t *__restrict__ tw_g, int nlines, int nh) {
    typedef typename C2<T>::t C;
    constexpr int R0 = zr_r0(N), R1 = zr_r1(N), G = zr_threads(N), LB = ZR_T / G, NB0 = N / R0, NB1 = N / R1;
    constexpr int I0 = (NB0 + G - 1) / G, I1 = (NB1 + G - 1) / G, LS = N + 1;
    static_assert(R0 * R1 == N && LB * G == ZR_T, "z transform plan");
    __shared__ C stw[N];
    extern __shared__ unsigned char smraw[];
    C *buf = (C *)smraw;  // [LB][LS]: the line between the stages
    // lines fastest across the threads: a half-warp reads 16 adjacent kx
    const int l = threadIdx.x % LB, t = threadIdx.x / LB;
    const long L = (long)blockIdx.x * LB + l;
    const bool act = L < nlines;
    long gb = 0;
    if (act) {
        const long j = L / nh, kx = L - j * nh;
        gb = j * N * nh + kx;
    }
    // first stage: every load issued before the twiddle table is staged
    C v[I0][R0];
#pragma unroll
    for (int it = 0; it < I0; it++) {
        const int j = t + it * G;
#pragma unroll
        for (int r = 0; r < R0; r++) v[it][r] = (act && j < NB0) ? spec[gb + (long)(j + r * NB0) * nh] : cmk<C>(0.0, 0.0);
    }
    for (int e = threadIdx.x; e < N; e += ZR_T) stw[e] = tw_g[e];
    __syncthreads();
    if constexpr (R1 == 1) {
        // one stage (N = R0): the DFT of the line, stored in natural order
#pragma unroll
        for (int it = 0; it < I0; it++) {
            reg_dft<R0, N>(v[it], stw);
            if (act && t + it * G < NB0) {
#pragma unroll
                for (int r = 0; r < R0; r++) spec[gb + (long)r * nh] = v[it][r];
            }
        }
    } else {
        C *bl = buf + l * LS;
#pragma unroll
        for (int it = 0; it < I0; it++) {
            const int j = t + it * G;
            if (j < NB0) {
                reg_dft<R0, N>(v[it], stw);
#pragma unroll
                for (int r = 0; r < R0; r++) bl[j * R0 + r] = v[it][r];
            }
        }
        __syncthreads();
        // second stage (Ns = R0 = NB1, so k = j, the twiddle step is 1 and
        // output r of butterfly j goes to j + r R0)
#pragma unroll
        for (int it = 0; it < I1; it++) {
            const int j = t + it * G;
            if (j < NB1) {
                C w[R1];
#pragma unroll
                for (int r = 0; r < R1; r++) w[r] = bl[j + r * NB1];
#pragma unroll
                for (int r = 1; r < R1; r++) w[r] = cmul(w[r], stw[r * j]);
                reg_dft<R1, N>(w, stw);
                if (act) {
#pragma unroll
                    for (int r = 0; r < R1; r++) spec[gb + (long)(j + r * R0) * nh] = w[r];
                }
            }
        }
    }
}

// z transforms of 384 and 512 points: three Stockham stages of radix 8, 8
// and 6 or 8 (register DFTs), the first loading and the last storing the
// spectrum directly; the middle stage works in place (every thread reads its
// butterflies' inputs, a barrier, then the writes).
constexpr int zr3_r(int n, int s) { return n == 384 ? (s < 2 ? 8 : 6) : (n == 512 ? 8 : 0); }
constexpr int ZR3_G = 32;  // threads per line (two or fewer butterflies of each stage per thread)

template <typename T, int N>
__global__ void __launch_bounds__(ZR_T) k_fft_zr3(typename C2<T>::t *__restrict__ spec,
                                                  const typename C2<T>::t *__restrict__ tw_g, int nlines, int nh) {
    typedef typename C2<T>::t C;
    constexpr int R0 = zr3_r(N, 0), R1 = zr3_r(N, 1), R2 = zr3_r(N, 2), G = ZR3_G, LB = ZR_T / G;
    constexpr int NB0 = N / R0, NB1 = N / R1, NB2 = N / R2, NS1 = R0, NS2 = R0 * R1, ST1 = N / (R0 * R1);
    constexpr int I0 = (NB0 + G - 1) / G, I1 = (NB1 + G - 1) / G, I2 = (NB2 + G - 1) / G, LS = N + 1;
    static_assert(R0 * R1 * R2 == N && NB2 == NS2, "z transform plan");
    __shared__ C stw[N];
    extern __shared__ unsigned char smraw[];
    // lines fastest across the threads: a half-warp reads 16 adjacent kx
    const int l = threadIdx.x % LB, t = threadIdx.x / LB;
    const long L = (long)blockIdx.x * LB + l;
    const bool act = L < nlines;
    long gb = 0;
    if (act) {
        const long j = L / nh, kx = L - j * nh;
        gb = j * N * nh + kx;
    }
    C *bl = (C *)smraw + l * LS;
    {
        C v[I0][R0];
#pragma unroll
        for (int it = 0; it < I0; it++) {
            const int j = t + it * G;
#pragma unroll
            for (int r = 0; r < R0; r++)
                v[it][r] = (act && j < NB0) ? spec[gb + (long)(j + r * NB0) * nh] : cmk<C>(0.0, 0.0);
        }
        for (int e = threadIdx.x; e < N; e += ZR_T) stw[e] = tw_g[e];
        __syncthreads();
#pragma unroll
        for (int it = 0; it < I0; it++) {
            const int j = t + it * G;
            if (j < NB0) {
                reg_dft<R0, N>(v[it], stw);
#pragma unroll
                for (int r = 0; r < R0; r++) bl[j * R0 + r] = v[it][r];
            }
        }
    }
    __syncthreads();
    {
        C w[I1][R1];
#pragma unroll
        for (int it = 0; it < I1; it++) {
            const int j = t + it * G, k = j % NS1;
            if (j < NB1) {
#pragma unroll
                for (int r = 0; r < R1; r++) w[it][r] = bl[j + r * NB1];
#pragma unroll
                for (int r = 1; r < R1; r++) w[it][r] = cmul(w[it][r], stw[r * k * ST1]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < I1; it++) {
            const int j = t + it * G, k = j % NS1;
            if (j < NB1) {
                reg_dft<R1, N>(w[it], stw);
                const int d = (j / NS1) * NS1 * R1 + k;
#pragma unroll
                for (int r = 0; r < R1; r++) bl[d + r * NS1] = w[it][r];
            }
        }
    }
    __syncthreads();
    // last stage: Ns = NB2, so k = j, the twiddle step is 1 and output r of
    // butterfly j goes to j + r NS2
#pragma unroll
    for (int it = 0; it < I2; it++) {
        const int j = t + it * G;
        if (j < NB2) {
            C w[R2];
#pragma unroll
            for (int r = 0; r < R2; r++) w[r] = bl[j + r * NB2];
#pragma unroll
            for (int r = 1; r < R2; r++) w[r] = cmul(w[r], stw[r * j]);
            reg_dft<R2, N>(w, stw);
            if (act) {
#pragma unroll
                for (int r = 0; r < R2; r++) spec[gb + (long)(j + r * NS2) * nh] = w[r];
            }
        }
    }
}

template <typename T, int N>
static size_t zr3_smem() {
    return (size_t)(ZR_T / ZR3_G) * (N + 1) * sizeof(typename C2<T>::t);
}

template <typename T, int N>
static size_t zr_smem() {
    return zr_r1(N) > 1 ? (size_t)(ZR_T / zr_threads(N)) * (N + 1) * sizeof(typename C2<T>::t) : 0;
}

// ---------------------------------------------------------------------------
// x transforms of the compile-time lengths up to 256 with the same two-stage
// plan (the forward one with the divergence fused, projection.f90:40-87; the
// inverse one into phi, :116-120).  The first stage of the forward transform
// forms its R0 divergences straight from U, V, W, the second stage of the
// inverse one stores phi directly.  A line sits in shared memory with one
// padding element after every R0 (position x at x + x / R0): the first
// stage's butterflies store R0 adjacent elements each, and with the padding
// both stages' accesses fall in distinct banks.
// ---------------------------------------------------------------------------
// radix of stage s of the x transforms' plan (1: no such stage): the two
// stages of the z plans up to 256 points, three for 384 and 512
constexpr int xr_r(int n, int s) {
    return zr_r0(n) > 0 ? (s == 0 ? zr_r0(n) : (s == 1 ? zr_r1(n) : 1)) : (zr3_r(n, 0) > 0 ? zr3_r(n, s) : 0);
}
// threads per line of the inverse x transform
constexpr int xr_threads(int n) { return zr_r0(n) > 0 ? zr_threads(n) : 32; }
template <int N> __device__ __forceinline__ int xr_pos(int x) { return x + x / xr_r(N, 0); }
template <int N> constexpr int xr_ls() { return N + N / xr_r(N, 0); }

// A middle Stockham stage (span NS, radix R) of a padded line in place:
// every thread reads its butterflies' inputs and applies the twiddles, a
// barrier, then the DFTs and the writes (G threads per line, thread t).
template <int N, int R, int NS, int G, typename C>
__device__ __forceinline__ void xr_mid_stage(C *bl, const C *stw, int t) {
    constexpr int NB = N / R, I = (NB + G - 1) / G, ST = N / (NS * R);
    C w[I][R];
#pragma unroll
    for (int it = 0; it < I; it++) {
        const int j = t + it * G, k = j % NS;
        if (j < NB) {
#pragma unroll
            for (int r = 0; r < R; r++) w[it][r] = bl[xr_pos<N>(j + r * NB)];
#pragma unroll
            for (int r = 1; r < R; r++) w[it][r] = cmul(w[it][r], stw[r * k * ST]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < I; it++) {
        const int j = t + it * G, k = j % NS;
        if (j < NB) {
            reg_dft<R, N>(w[it], stw);
            const int d = (j / NS) * NS * R + k;
#pragma unroll
            for (int r = 0; r < R; r++) bl[xr_pos<N>(d + r * NS)] = w[it][r];
        }
    }
}

// Forward: the divergence of the packed line pair is formed by 32 threads
// per pair (x positions t + 32 e, every load of a thread issued before the
// arithmetic) into the padded line, then the two register stages (the first
// stage reads all its butterflies' inputs before any of them is stored back)
// and the split into the two half spectra.
constexpr int XR_FT = 32;  // threads per line pair of the forward x transform

template <typename T, int N>
__global__ void __launch_bounds__(ZR_T) k_fwd_xr(GeoT<T> g, Fld<T> U, Fld<T> V, Fld<T> W, typename C2<T>::t *spec,
                                                 const typename C2<T>::t *__restrict__ tw_g, RSp rs) {
    typedef typename C2<T>::t C;
    constexpr int R0 = xr_r(N, 0), R1 = xr_r(N, 1), R2 = xr_r(N, 2), G = XR_FT, LP = ZR_T / G, NB0 = N / R0;
    constexpr int RL = R2 > 1 ? R2 : R1, NSL = N / RL, NBL = N / RL;  // the last stage (span NSL)
    constexpr int I0 = (NB0 + G - 1) / G, IL = (NBL + G - 1) / G, LS = xr_ls<N>(), NH = N / 2 + 1;
    constexpr int NPT = (N + G - 1) / G, XB = NPT < 3 ? NPT : 3;
    __shared__ C stw[N];
    extern __shared__ unsigned char smraw[];
    const int lp = threadIdx.x / G, t = threadIdx.x % G;
    const int nym = g.nym, nzp = g.nzp;
    const long pair = (long)blockIdx.x * LP + lp;
    const bool act = pair < (long)nym * (nzp / 2);
    int j = 2, k = 2;
    if (act) {
        j = (int)(pair % nym) + 2;
        k = (int)(pair / nym) * 2 + 2;
    }
    C *bl = (C *)smraw + lp * LS;
    // divergences of lines k (real part) and k+1 (imaginary part); the x and
    // z neighbours below the first interior index through the periodic wrap
    // (U(1) = U(nxp+1), W(k=1) = W(nzp+1))
    const int km = k == 2 ? nzp + 1 : k - 1, k1 = k + 1;
    if (act) {
        T ry = T(0), rz0 = T(0), rz1 = T(0);
        if constexpr (sizeof(T) == 4) {
            ry = rs.ry[j];
            rz0 = rs.rz[k];
            rz1 = rs.rz[k + 1];
        }
#pragma unroll
        for (int e0 = 0; e0 < NPT; e0 += XB) {
            T ua[XB], uam[XB], ub[XB], ubm[XB], va[XB], vam[XB], vb[XB], vbm[XB], wa[XB], wb[XB], wm[XB];
#pragma unroll
            for (int b = 0; b < XB; b++) {
                const int x = t + (e0 + b) * G, i = x + 2, im = i == 2 ? N + 1 : i - 1;
                if (e0 + b < NPT && x < N) {
                    ua[b] = U(i, j, k); uam[b] = U(im, j, k); ub[b] = U(i, j, k1); ubm[b] = U(im, j, k1);
                    va[b] = V(i, j, k); vam[b] = V(i, j - 1, k); vb[b] = V(i, j, k1); vbm[b] = V(i, j - 1, k1);
                    wa[b] = W(i, j, k); wb[b] = W(i, j, k1); wm[b] = W(i, j, km);
                }
            }
#pragma unroll
            for (int b = 0; b < XB; b++) {
                const int x = t + (e0 + b) * G, i = x + 2;
                if (e0 + b < NPT && x < N) {
                    C z;
                    if constexpr (sizeof(T) == 4) {
                        const T rx = rs.rx[i];
                        z.x = (ua[b] - uam[b]) * rx + (va[b] - vam[b]) * ry + (wa[b] - wm[b]) * rz0;
                        z.y = (ub[b] - ubm[b]) * rx + (vb[b] - vbm[b]) * ry + (wb[b] - wa[b]) * rz1;
                    } else {
                        z.x = (ua[b] - uam[b]) / (g.x[i] - g.x[i - 1]) + (va[b] - vam[b]) / (g.y[j] - g.y[j - 1]) +
                              (wa[b] - wm[b]) / (g.z[k] - g.z[k - 1]);
                        z.y = (ub[b] - ubm[b]) / (g.x[i] - g.x[i - 1]) + (vb[b] - vbm[b]) / (g.y[j] - g.y[j - 1]) +
                              (wb[b] - wa[b]) / (g.z[k1] - g.z[k1 - 1]);
                    }
                    bl[xr_pos<N>(x)] = z;
                }
            }
        }
    }
    for (int e = threadIdx.x; e < N; e += ZR_T) stw[e] = tw_g[e];
    __syncthreads();
    // first stage: inputs jb + NB0 r, outputs jb R0 + r (read all, then store)
    C v[I0][R0];
#pragma unroll
    for (int it = 0; it < I0; it++) {
        const int jb = t + it * G;
        if (jb < NB0) {
#pragma unroll
            for (int r = 0; r < R0; r++) v[it][r] = bl[xr_pos<N>(jb + NB0 * r)];
            reg_dft<R0, N>(v[it], stw);
        }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < I0; it++) {
        const int jb = t + it * G;
        if (jb < NB0) {
#pragma unroll
            for (int r = 0; r < R0; r++) bl[xr_pos<N>(jb * R0 + r)] = v[it][r];
        }
    }
    if constexpr (R2 > 1) {
        __syncthreads();
        xr_mid_stage<N, R1, R0, G>(bl, stw, t);
    }
    if constexpr (R1 > 1) {
        __syncthreads();
        // last stage in place (span NSL = NBL, twiddle step 1): butterfly
        // jb reads and writes jb + r NSL
#pragma unroll
        for (int it = 0; it < IL; it++) {
            const int jb = t + it * G;
            if (jb < NBL) {
                C w[RL];
#pragma unroll
                for (int r = 0; r < RL; r++) w[r] = bl[xr_pos<N>(jb + r * NSL)];
#pragma unroll
                for (int r = 1; r < RL; r++) w[r] = cmul(w[r], stw[r * jb]);
                reg_dft<RL, N>(w, stw);
#pragma unroll
                for (int r = 0; r < RL; r++) bl[xr_pos<N>(jb + r * NSL)] = w[r];
            }
        }
    }
    __syncthreads();
    if (!act) return;
    // the two half spectra of the packed lines: Z(q) = A(q) + i B(q)
    C *o0 = spec + ((long)(j - 2) * nzp + (k - 2)) * NH, *o1 = spec + ((long)(j - 2) * nzp + (k - 1)) * NH;
    for (int q = t; q < NH; q += G) {
        const C Zk = bl[xr_pos<N>(q)], Zc = cconj(bl[xr_pos<N>((N - q) % N)]);
        C A, B;
        A.x = T(0.5) * (Zk.x + Zc.x);
        A.y = T(0.5) * (Zk.y + Zc.y);
        B.x = T(0.5) * (Zk.y - Zc.y);  // (Zk - Zc)/(2i)
        B.y = -T(0.5) * (Zk.x - Zc.x);
        o0[q] = A;
        o1[q] = B;
    }
}

template <typename T, int N>
__global__ void __launch_bounds__(ZR_T) k_inv_xr(const typename C2<T>::t *__restrict__ spec, T *__restrict__ phi,
                                                 const typename C2<T>::t *__restrict__ tw_g, int nym, int nzp, T scale) {
    typedef typename C2<T>::t C;
    constexpr int R0 = xr_r(N, 0), R1 = xr_r(N, 1), R2 = xr_r(N, 2), G = xr_threads(N), LP = ZR_T / G, NB0 = N / R0;
    constexpr int RL = R2 > 1 ? R2 : R1, NSL = N / RL, NBL = N / RL;  // the last stage (span NSL)
    constexpr int I0 = (NB0 + G - 1) / G, IL = (NBL + G - 1) / G, LS = xr_ls<N>(), NH = N / 2 + 1;
    __shared__ C stw[N];
    extern __shared__ unsigned char smraw[];
    const int lp = threadIdx.x / G, t = threadIdx.x % G;
    const long pair = (long)blockIdx.x * LP + lp;
    const bool act = pair < (long)nym * (nzp / 2);
    int jj = 0, kk = 0;
    if (act) {
        jj = (int)(pair % nym);
        kk = (int)(pair / nym) * 2;
    }
    const C *s0 = spec + ((long)jj * nzp + kk) * NH, *s1 = spec + ((long)jj * nzp + kk + 1) * NH;
    // first stage: z(q) = A(q) + i B(q) from the two half spectra
    // (conjugate symmetric above NH, real at q = 0 and N/2)
    C v[I0][R0];
#pragma unroll
    for (int it = 0; it < I0; it++) {
        const int jb = t + it * G;
#pragma unroll
        for (int r = 0; r < R0; r++) {
            C z = cmk<C>(0.0, 0.0);
            if (act && jb < NB0) {
                const int q = jb + NB0 * r, src = q < NH ? q : N - q;
                C a0 = s0[src], b0 = s1[src];
                if (q < NH) {
                    if (q == 0 || 2 * q == N) { a0.y = 0; b0.y = 0; }
                } else {
                    a0 = cconj(a0);
                    b0 = cconj(b0);
                }
                z.x = a0.x - b0.y;
                z.y = a0.y + b0.x;
            }
            v[it][r] = z;
        }
    }
    for (int e = threadIdx.x; e < N; e += ZR_T) stw[e] = tw_g[e];
    __syncthreads();
    T *p0 = phi + (long)N * (jj + (long)nym * kk), *p1 = phi + (long)N * (jj + (long)nym * (kk + 1));
    if constexpr (R1 == 1) {
        reg_dft<R0, N>(v[0], stw);
        if (act) {
#pragma unroll
            for (int r = 0; r < R0; r++) {
                p0[r] = v[0][r].x * scale;
                p1[r] = v[0][r].y * scale;
            }
        }
    } else {
        C *bl = (C *)smraw + lp * LS;
#pragma unroll
        for (int it = 0; it < I0; it++) {
            const int jb = t + it * G;
            if (jb < NB0) {
                reg_dft<R0, N>(v[it], stw);
#pragma unroll
                for (int r = 0; r < R0; r++) bl[xr_pos<N>(jb * R0 + r)] = v[it][r];
            }
        }
        __syncthreads();
        if constexpr (R2 > 1) {
            xr_mid_stage<N, R1, R0, G>(bl, stw, t);
            __syncthreads();
        }
        // last stage (span NSL = NBL, twiddle step 1): phi stored directly
#pragma unroll
        for (int it = 0; it < IL; it++) {
            const int jb = t + it * G;
            if (jb < NBL) {
                C w[RL];
#pragma unroll
                for (int r = 0; r < RL; r++) w[r] = bl[xr_pos<N>(jb + r * NSL)];
#pragma unroll
                for (int r = 1; r < RL; r++) w[r] = cmul(w[r], stw[r * jb]);
                reg_dft<RL, N>(w, stw);
                if (act) {
#pragma unroll
                    for (int r = 0; r < RL; r++) {
                        p0[jb + r * NSL] = w[r].x * scale;
                        p1[jb + r * NSL] = w[r].y * scale;
                    }
                }
            }
        }
    }
}

template <typename T, int N>
static size_t xr_smem() {
    return xr_r(N, 1) > 1 ? (size_t)(ZR_T / xr_threads(N)) * xr_ls<N>() * sizeof(typename C2<T>::t) : 0;
}
template <typename T, int N>
static size_t xr_fwd_smem() {
    return (size_t)(ZR_T / XR_FT) * xr_ls<N>() * sizeof(typename C2<T>::t);
}

// ---------------------------------------------------------------------------
// Tridiagonal solve per mode m = kz*nh + kx along j (projection.f90:90-113).
// The matrices D(j) = Dyy(j,j) + kxx + kzz (with D(2)*1.5 for the (0,0)
// mode) never change, so zgtsv's elimination -- pivot choices, multipliers
// and the final U factor -- is done once on the host (tri_factor) and a
// solve only replays its right-hand-side operations:
//   fwd q: no pivot: b[q+1] -= m_q b[q]
//          pivot:    (b[q], b[q+1]) <- (b[q+1], b[q] - m_q b[q+1])
//   back:  b[q] = (b[q] - du_q b[q+1] - dl_q b[q+2]) * rd_q
// Spectrum and factors are stored [row][mode].
// ---------------------------------------------------------------------------
struct TriFac {
    const double *m, *rd, *du, *dl;  // [nym][NM]
    const unsigned char *piv;        // [nym][NM]
};

// FP64 replay, one 32-thread block per mode (all modes, or the modes of
// `list`): the warp stages the mode's right-hand side and factors in shared
// memory with independent loads, then lane 0 runs the serial recurrence out
// of shared memory.
template <typename T>
__global__ void __launch_bounds__(32) k_tri_mode(typename C2<T>::t *__restrict__ spec, TriFac f, int nym, long NM,
                                                 const int *__restrict__ list) {
    typedef typename C2<T>::t C;
    extern __shared__ double tsm[];
    double *br = tsm, *bi = br + nym, *fm = bi + nym, *frd = fm + nym, *fdu = frd + nym, *fdl = fdu + nym;
    unsigned char *fp = (unsigned char *)(fdl + nym);
    const long mo = list ? list[blockIdx.x] : blockIdx.x;
    for (int q = threadIdx.x; q < nym; q += 32) {
        const long o = (long)q * NM + mo;
        C v = spec[o];
        br[q] = v.x;
        bi[q] = v.y;
        fm[q] = f.m[o];
        frd[q] = f.rd[o];
        fdu[q] = f.du[o];
        fdl[q] = f.dl[o];
        fp[q] = f.piv[o];
    }
    __syncwarp();
    if (threadIdx.x == 0) {
        double r0 = br[0], i0 = bi[0];
        for (int q = 0; q < nym - 1; q++) {
            double nre = br[q + 1], nim = bi[q + 1], m = fm[q];
            if (fp[q]) {
                br[q] = nre;
                bi[q] = nim;
                nre = r0 - m * nre;
                nim = i0 - m * nim;
            } else {
                br[q] = r0;
                bi[q] = i0;
                nre = nre - m * r0;
                nim = nim - m * i0;
            }
            r0 = nre;
            i0 = nim;
        }
        double x1r = r0 * frd[nym - 1], x1i = i0 * frd[nym - 1], x2r = 0.0, x2i = 0.0;
        br[nym - 1] = x1r;
        bi[nym - 1] = x1i;
        for (int q = nym - 2; q >= 0; q--) {
            double yr = (br[q] - fdu[q] * x1r - fdl[q] * x2r) * frd[q];
            double yi = (bi[q] - fdu[q] * x1i - fdl[q] * x2i) * frd[q];
            br[q] = yr;
            bi[q] = yi;
            x2r = x1r;
            x2i = x1i;
            x1r = yr;
            x1i = yi;
        }
    }
    __syncwarp();
    for (int q = threadIdx.x; q < nym; q += 32) spec[(long)q * NM + mo] = cmk<C>(br[q], bi[q]);
}

static size_t tri_mode_smem(int nym) { return (size_t)nym * (6 * sizeof(double) + 1); }

// The tridiagonal systems of many channels in one launch (ensembles): the
// FP64 replay of k_tri_mode (zgtsv's elimination with its recorded pivots)
// with one thread per (member, mode).  Modes of a member are adjacent in
// memory ([row][mode]), so a warp's loads of one row are coalesced; warps
// never straddle members (each member's modes start a new 32-block).  The
// eliminated right-hand side is kept in FP64 scratch [row][mode], so FP32
// spectra (split-path members) are solved in FP64 throughout and FP64
// members bit for bit as k_tri_mode.
constexpr int TRI_BATCH_T = 64;

__global__ void __launch_bounds__(TRI_BATCH_T) k_tri_batch(const TriMember *__restrict__ tab, int nmem) {
    const long gb = blockIdx.x;
    int lo = 0, hi = nmem - 1;
    while (lo < hi) {  // last member whose first block <= gb
        const int mid = (lo + hi + 1) >> 1;
        if (tab[mid].first <= gb) lo = mid;
        else hi = mid - 1;
    }
    const TriMember t = tab[lo];
    const long mo = (gb - t.first) * TRI_BATCH_T + threadIdx.x, NM = t.NM;
    if (mo >= NM) return;
    const int nym = t.nym;
    double2 *sc = t.scratch;
    auto rd_spec = [&](long o) -> double2 {
        if (t.esz == 4) {
            const float2 v = ((const float2 *)t.spec)[o];
            return make_double2(v.x, v.y);
        }
        return ((const double2 *)t.spec)[o];
    };
    double2 r0 = rd_spec(mo);
    for (int q = 0; q < nym - 1; q++) {
        const long o = (long)q * NM + mo;
        double2 nx = rd_spec(o + NM);
        const double m = t.m[o];
        if (t.piv[o]) {
            sc[o] = nx;
            nx = make_double2(r0.x - m * nx.x, r0.y - m * nx.y);
        } else {
            sc[o] = r0;
            nx = make_double2(nx.x - m * r0.x, nx.y - m * r0.y);
        }
        r0 = nx;
    }
    const long ol = (long)(nym - 1) * NM + mo;
    double x1r = r0.x * t.rd[ol], x1i = r0.y * t.rd[ol], x2r = 0.0, x2i = 0.0;
    auto wr_spec = [&](long o, double a, double b) {
        if (t.esz == 4) ((float2 *)t.spec)[o] = make_float2((float)a, (float)b);
        else ((double2 *)t.spec)[o] = make_double2(a, b);
    };
    wr_spec(ol, x1r, x1i);
    for (int q = nym - 2; q >= 0; q--) {
        const long o = (long)q * NM + mo;
        const double2 b = sc[o];
        const double du = t.du[o], dl = t.dl[o], rdq = t.rd[o];
        const double yr = (b.x - du * x1r - dl * x2r) * rdq;
        const double yi = (b.y - du * x1i - dl * x2i) * rdq;
        wr_spec(o, yr, yi);
        x2r = x1r;
        x2i = x1i;
        x1r = yr;
        x1i = yi;
    }
}

TriMember tri_member(const cf_ctx *ctx) {
    TriMember t;
    const long NM = (long)ctx->nzp * ctx->nxh;
    const size_t nf = (size_t)ctx->nym * NM;
    t.spec = ctx->spec;
    t.m = ctx->tri_fac;
    t.rd = ctx->tri_fac + nf;
    t.du = ctx->tri_fac + 2 * nf;
    t.dl = ctx->tri_fac + 3 * nf;
    t.piv = ctx->tri_piv;
    t.nym = ctx->nym;
    t.esz = ctx->esz;
    t.NM = NM;
    t.first = 0;
    return t;
}

long tri_batch_blocks(long NM) { return (NM + TRI_BATCH_T - 1) / TRI_BATCH_T; }

int launch_tri_batch(cudaStream_t st, const TriMember *dtab, int nmem, long total_blocks) {
    k_tri_batch<<<(unsigned)total_blocks, TRI_BATCH_T, 0, st>>>(dtab, nmem);
    return cudaGetLastError() == cudaSuccess ? 0 : CF_ERR_CUDA;
}


// Split path, one launch for every mode.
//  * Blocks nlist.. : MB modes whose elimination never pivots, one thread each
//    (adjacent in memory): zgtsv's no-pivot replay
//      b[q+1] -= m_q b[q];  b[q] = (b[q] - du_q b[q+1]) rd_q
//    in FP32 with the FP64 factors rounded once.  The block copies every row
//    of its modes' right-hand sides and factors into shared memory with
//    asynchronous copies (all in flight at once), then each thread runs its
//    recurrence out of shared memory.
//  * Blocks 0..nlist-1: one mode whose elimination pivots (the lowest
//    wavenumbers, condition numbers up to ~1e5).  An FP32 replay of the full
//    pivoting elimination is refined once against the FP64 residual b - A x
//    (rows in parallel, x accumulated in FP64): the refined error (~1e-6
//    relative for the (0,0) mode, less elsewhere) is near the FP32 rounding
//    of the stored result, without a serial FP64 chain (dependent FP64
//    operations are slow on this GPU).  The block's first warp does the
//    work; its lane 0 runs the recurrences.
struct TriSplit {
    const float *l, *ru, *du;        // FP32 no-pivot factors [nym][NM], du [nym]
    const unsigned char *flag;       // [NM] 1: the mode pivots
    const int *list;                 // flagged modes
    int nlist;
    const double *Dd, *Dl, *Du;      // Dyy rows (nym each): diagonal, A(q+1,q), A(q,q+1)
    const double *kxx, *kzz;
    int nh;
};

// col(q): the mode's right-hand side / solution at row q; one warp, lane =
// its lane; the scratch smraw holds tri_refined_smem(nym) bytes.
// col(q): the mode's right-hand side / solution at row q; one warp, lane =
// its lane; the scratch smraw holds tri_refined_smem(nym) bytes.
//
// Each FP32 replay runs across the warp as a segmented scan (lane L takes a
// contiguous block of steps).  Forward, step k with carry c (the current
// value of row k): no interchange keeps c in row k and carries
// w_{k+1} - m_k c; an interchange puts w_{k+1} in row k and carries
// c - m_k w_{k+1} -- in both cases c' = alpha c + beta, an affine map
// (|alpha| <= 1 by the pivoting), composed per lane, scanned over the lanes
// and replayed with the true carry.  Backward, x_q = rd_q o_q -
// (rd du)_q x_{q+1} - (rd dl)_q x_{q+2}: the affine map of the state
// (x_{q+1}, x_{q+2}) -> (x_q, x_{q+1}) with a 2x2 matrix, scanned the same way
// from the last row (state 0 beyond it).
template <typename Col>
__device__ void tri_refined_col(Col col, const TriFac &f, const TriSplit &ts, int nym, long NM, long mo,
                                unsigned char *smraw, int lane) {
    double *b_re = (double *)smraw, *b_im = b_re + nym, *x_re = b_im + nym, *x_im = x_re + nym;
    float *w_re = (float *)(x_im + nym), *w_im = w_re + nym, *o_re = w_im + nym, *o_im = o_re + nym,
          *fm = o_im + nym, *frd = fm + nym, *fdu = frd + nym, *fdl = fdu + nym;
    unsigned char *fp = (unsigned char *)(fdl + nym);
    const int nt = 32;
    const unsigned FULL = 0xffffffffu;
    const int kx = (int)(mo % ts.nh), kz = (int)(mo / ts.nh);
    const double k2 = ts.kxx[kx] + ts.kzz[kz];
    for (int q = lane; q < nym; q += nt) {
        const long o = (long)q * NM + mo;
        const float2 v = col(q);
        b_re[q] = v.x;
        b_im[q] = v.y;
        x_re[q] = 0.0;
        x_im[q] = 0.0;
        w_re[q] = v.x;
        w_im[q] = v.y;
        // back substitution coefficients scaled by 1/d; zero beyond the band
        fm[q] = (float)f.m[o];
        frd[q] = (float)f.rd[o];
        fdu[q] = q < nym - 1 ? (float)(f.rd[o] * f.du[o]) : 0.f;
        fdl[q] = q < nym - 2 ? (float)(f.rd[o] * f.dl[o]) : 0.f;
        fp[q] = f.piv[o];
    }
    __syncwarp();
    const int nf = nym - 1, SF = (nf + nt - 1) / nt, SB = (nym + nt - 1) / nt;
    const int k0 = min(lane * SF, nf), k1 = min(k0 + SF, nf);
    const int t0 = min(lane * SB, nym), t1 = min(t0 + SB, nym);
    for (int it = 0; it < 2; it++) {
        // ---- forward: steps k = 0 .. nym-2, carry c_0 = w_0
        {
            float A = 1.f, Br = 0.f, Bi = 0.f;
            for (int k = k0; k < k1; k++) {
                const float m = fm[k], wr = w_re[k + 1], wi = w_im[k + 1];
                const bool pv = fp[k] != 0;
                const float al = pv ? 1.f : -m;
                Br = al * Br + (pv ? -m * wr : wr);
                Bi = al * Bi + (pv ? -m * wi : wi);
                A = al * A;
            }
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const float Ap = __shfl_up_sync(FULL, A, d), Brp = __shfl_up_sync(FULL, Br, d),
                            Bip = __shfl_up_sync(FULL, Bi, d);
                if (lane >= d) {
                    Br = A * Brp + Br;
                    Bi = A * Bip + Bi;
                    A = A * Ap;
                }
            }
            const float pA = __shfl_up_sync(FULL, A, 1), pBr = __shfl_up_sync(FULL, Br, 1),
                        pBi = __shfl_up_sync(FULL, Bi, 1);
            const float c0r = w_re[0], c0i = w_im[0];
            float cr = lane ? pA * c0r + pBr : c0r, ci = lane ? pA * c0i + pBi : c0i;
            for (int k = k0; k < k1; k++) {
                const float m = fm[k], wr = w_re[k + 1], wi = w_im[k + 1];
                const bool pv = fp[k] != 0;
                const float orr = pv ? wr : cr, oi = pv ? wi : ci;
                o_re[k] = orr;
                o_im[k] = oi;
                cr = (pv ? cr : wr) - m * orr;
                ci = (pv ? ci : wi) - m * oi;
            }
            if (k1 == nf && k0 < k1) {  // the lane with the last step
                o_re[nf] = cr;
                o_im[nf] = ci;
            }
            if (nf == 0 && lane == 0) {
                o_re[0] = c0r;
                o_im[0] = c0i;
            }
        }
        __syncwarp();
        // ---- backward: steps t = 0 .. nym-1 on rows q = nym-1-t
        {
            float m00 = 1.f, m01 = 0.f, m10 = 0.f, m11 = 1.f, v0r = 0.f, v0i = 0.f, v1r = 0.f, v1i = 0.f;
            for (int t = t0; t < t1; t++) {
                const int q = nym - 1 - t;
                const float a = fdu[q], bq = fdl[q], r = frd[q];
                const float n00 = -a * m00 - bq * m10, n01 = -a * m01 - bq * m11;
                m10 = m00;
                m11 = m01;
                m00 = n00;
                m01 = n01;
                const float u0r = -a * v0r - bq * v1r + r * o_re[q], u0i = -a * v0i - bq * v1i + r * o_im[q];
                v1r = v0r;
                v1i = v0i;
                v0r = u0r;
                v0i = u0i;
            }
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const float p00 = __shfl_up_sync(FULL, m00, d), p01 = __shfl_up_sync(FULL, m01, d),
                            p10 = __shfl_up_sync(FULL, m10, d), p11 = __shfl_up_sync(FULL, m11, d);
                const float q0r = __shfl_up_sync(FULL, v0r, d), q0i = __shfl_up_sync(FULL, v0i, d),
                            q1r = __shfl_up_sync(FULL, v1r, d), q1i = __shfl_up_sync(FULL, v1i, d);
                if (lane >= d) {
                    // (M, v) after (P, p): (M P, M p + v)
                    const float n0r = m00 * q0r + m01 * q1r + v0r, n0i = m00 * q0i + m01 * q1i + v0i;
                    const float n1r = m10 * q0r + m11 * q1r + v1r, n1i = m10 * q0i + m11 * q1i + v1i;
                    const float a00 = m00 * p00 + m01 * p10, a01 = m00 * p01 + m01 * p11;
                    const float a10 = m10 * p00 + m11 * p10, a11 = m10 * p01 + m11 * p11;
                    m00 = a00; m01 = a01; m10 = a10; m11 = a11;
                    v0r = n0r; v0i = n0i; v1r = n1r; v1i = n1i;
                }
            }
            // carry in: the state after the lanes before (from state 0)
            const float s0r = __shfl_up_sync(FULL, v0r, 1), s0i = __shfl_up_sync(FULL, v0i, 1),
                        s1r = __shfl_up_sync(FULL, v1r, 1), s1i = __shfl_up_sync(FULL, v1i, 1);
            float x1r = lane ? s0r : 0.f, x1i = lane ? s0i : 0.f, x2r = lane ? s1r : 0.f, x2i = lane ? s1i : 0.f;
            for (int t = t0; t < t1; t++) {
                const int q = nym - 1 - t;
                const float a = fdu[q], bq = fdl[q], r = frd[q];
                const float yr = (r * o_re[q] - bq * x2r) - a * x1r, yi = (r * o_im[q] - bq * x2i) - a * x1i;
                w_re[q] = yr;
                w_im[q] = yi;
                x2r = x1r;
                x2i = x1i;
                x1r = yr;
                x1i = yi;
            }
        }
        __syncwarp();
        for (int q = lane; q < nym; q += nt) {
            x_re[q] += (double)w_re[q];
            x_im[q] += (double)w_im[q];
        }
        __syncwarp();
        if (it == 1) break;
        // residual of the original matrix (projection.f90:97-107) in FP64
        for (int q = lane; q < nym; q += nt) {
            double d = ts.Dd[q] + k2;
            if (q == 0 && kx == 0 && kz == 0) d = 1.5 * d;
            double ar = d * x_re[q], ai = d * x_im[q];
            if (q > 0) {
                ar += ts.Dl[q - 1] * x_re[q - 1];
                ai += ts.Dl[q - 1] * x_im[q - 1];
            }
            if (q < nym - 1) {
                ar += ts.Du[q] * x_re[q + 1];
                ai += ts.Du[q] * x_im[q + 1];
            }
            w_re[q] = (float)(b_re[q] - ar);
            w_im[q] = (float)(b_im[q] - ai);
        }
        __syncwarp();
    }
    for (int q = lane; q < nym; q += nt) col(q) = make_float2((float)x_re[q], (float)x_im[q]);
}

__host__ __device__ static inline size_t tri_refined_smem(int nym) {
    return (size_t)nym * (4 * sizeof(double) + 8 * sizeof(float) + 1);
}

// Bulk modes: the no-pivot replay y_j = b_j - m_{j-1} y_{j-1},
// x_j = (y_j - du_j x_{j+1}) rd_j split over P = blockDim.y segments of
// TRI_RS rows, one thread per (mode, segment), 32 adjacent modes per warp.
// Each segment runs both first-order recurrences locally from a zero carry
// while tracking the carry's coefficient (a product of |m| < 1 or
// |du rd| < 1: the matrices are diagonally dominant); the segment-end values
// are combined across segments through shared memory and each row is then
// corrected by coefficient x true carry.
template <int TRI_RS>
__device__ void tri_bulk_segmented(float2 *__restrict__ spec, const TriSplit &ts, int nym, long NM, int blk,
                                   unsigned char *smraw) {
    const int lane = threadIdx.x, p = threadIdx.y, P = blockDim.y;
    const long mo = (long)blk * 32 + lane;
    const bool act = mo < NM && !ts.flag[mo];
    float2 *sY = (float2 *)smraw;      // [P][32] segment-end values
    float *sC = (float *)(sY + P * 32);  // [P][32] their carry coefficients
    const int j0 = p * TRI_RS;
    float2 y[TRI_RS];
    float c[TRI_RS], rd[TRI_RS], g[TRI_RS];
    // loads: right-hand side, multiplier of the row above, 1/d, du
#pragma unroll
    for (int r = 0; r < TRI_RS; r++) {
        const int j = j0 + r;
        y[r] = make_float2(0.f, 0.f);
        c[r] = 0.f;
        rd[r] = 0.f;
        g[r] = 0.f;
        if (act && j < nym) {
            const long o = (long)j * NM + mo;
            y[r] = spec[o];
            c[r] = j > 0 ? ts.l[o - NM] : 0.f;  // m_{j-1}
            rd[r] = ts.ru[o];
            g[r] = ts.du[j];
        }
    }
    // forward, local: y_j -= m_{j-1} y_{j-1}; coefficient of the incoming carry
    {
        float2 yp = make_float2(0.f, 0.f);
        float cp = 1.f;
#pragma unroll
        for (int r = 0; r < TRI_RS; r++) {
            const float m = c[r];
            y[r].x = y[r].x - m * yp.x;
            y[r].y = y[r].y - m * yp.y;
            cp = -m * cp;
            c[r] = cp;
            yp = y[r];
        }
        sY[p * 32 + lane] = yp;
        sC[p * 32 + lane] = cp;
    }
    __syncthreads();
    {
        float2 carry = make_float2(0.f, 0.f);  // true y at the row before this segment
        for (int q = 0; q < p; q++) {
            const float2 Yq = sY[q * 32 + lane];
            const float Cq = sC[q * 32 + lane];
            carry.x = Yq.x + Cq * carry.x;
            carry.y = Yq.y + Cq * carry.y;
        }
#pragma unroll
        for (int r = 0; r < TRI_RS; r++) {
            y[r].x += c[r] * carry.x;
            y[r].y += c[r] * carry.y;
        }
    }
    __syncthreads();
    // backward, local: x_j = y_j rd_j - du_j rd_j x_{j+1}
    {
        float2 xn = make_float2(0.f, 0.f);
        float en = 1.f;
#pragma unroll
        for (int r = TRI_RS - 1; r >= 0; r--) {
            const float gg = -g[r] * rd[r];
            float2 x;
            x.x = (y[r].x - g[r] * xn.x) * rd[r];
            x.y = (y[r].y - g[r] * xn.y) * rd[r];
            en = gg * en;
            y[r] = x;
            c[r] = en;
            xn = x;
        }
        sY[p * 32 + lane] = xn;  // x at the segment's first row
        sC[p * 32 + lane] = en;
    }
    __syncthreads();
    {
        float2 carry = make_float2(0.f, 0.f);  // true x at the row after this segment
        for (int q = P - 1; q > p; q--) {
            const float2 Xq = sY[q * 32 + lane];
            const float Eq = sC[q * 32 + lane];
            carry.x = Xq.x + Eq * carry.x;
            carry.y = Xq.y + Eq * carry.y;
        }
#pragma unroll
        for (int r = 0; r < TRI_RS; r++) {
            const int j = j0 + r;
            if (act && j < nym) {
                float2 x = y[r];
                x.x += c[r] * carry.x;
                x.y += c[r] * carry.y;
                spec[(long)j * NM + mo] = x;
            }
        }
    }
}

// The split-path solve in one launch: blocks 0 .. npb-1 solve the pivoting
// modes, one per warp (pw warps per block), their replays warp-wide so that
// they finish within the first wave of the bulk blocks; the remaining blocks
// take 32 bulk modes x P segments of RS rows each.
constexpr size_t TRI_SPLIT_SMEM = 96 * 1024;  // shared memory of a block at most
template <int RS>
__global__ void __launch_bounds__(512) k_tri_split(float2 *__restrict__ spec, TriFac f, TriSplit ts, int nym, long NM,
                                                   int npb, int pw) {
    extern __shared__ float2 t32[];
    if ((int)blockIdx.x < npb) {
        const int w = threadIdx.y, e = blockIdx.x * pw + w;
        if (w >= pw || e >= ts.nlist) return;
        const long mo = ts.list[e];
        auto col = [&](int q) -> float2 & { return spec[(long)q * NM + mo]; };
        tri_refined_col(col, f, ts, nym, NM, mo,
                        (unsigned char *)t32 + (size_t)w * ((tri_refined_smem(nym) + 15) & ~(size_t)15),
                        (int)threadIdx.x);
        return;
    }
    tri_bulk_segmented<RS>(spec, ts, nym, NM, blockIdx.x - npb, (unsigned char *)t32);
}

// rows per segment: 16 up to 256 rows (at most 16 segments), else 32
static int tri_split_rs(int nym) { return nym <= 256 ? 16 : 32; }

// ---------------------------------------------------------------------------
// Inverse x: two half spectra -> one complex sequence -> FFT (+) -> real
// lines (j,k), (j,k+1) into phi (canonical), scaled by 1/(nxp*nzp)
// (projection.f90:116-120).
// ---------------------------------------------------------------------------
template <typename T, int N>
__global__ void k_inv_x(const typename C2<T>::t *spec, T *phi, FftPlan pl, const typename C2<T>::t *tw_g, int nym, int nzp,
                        int LP, T scale) {
    typedef typename C2<T>::t C;
    extern __shared__ unsigned char smraw[];
    C *sm = (C *)smraw;
    const int n = N > 0 ? N : pl.n, G = N > 0 ? fft_x_threads(N) : blockDim.x / LP, nh = n / 2 + 1;
    const C *tw = stage_twiddles<N, C>(tw_g, sm + (long)LP * 2 * n);
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
    if (active && N > 0) {
        // compile-time length: every load of the thread issued before the
        // first store to shared memory
        constexpr int GX = fft_x_threads(N > 0 ? N : 16), NPT = N > 0 ? N / GX : 1;
        const C *s0 = spec + ((long)jj * nzp + kk) * nh, *s1 = spec + ((long)jj * nzp + kk + 1) * nh;
        C A[NPT], B[NPT];
#pragma unroll
        for (int e = 0; e < NPT; e++) {
            const int q = tid + e * GX, src = q < nh ? q : n - q;
            A[e] = s0[src];
            B[e] = s1[src];
        }
#pragma unroll
        for (int e = 0; e < NPT; e++) {
            const int q = tid + e * GX;
            C a0 = A[e], b0 = B[e];
            if (q < nh) {
                if (q == 0 || 2 * q == n) { a0.y = 0; b0.y = 0; }
            } else {
                a0 = cconj(a0);
                b0 = cconj(b0);
            }
            C z;  // A + i B
            z.x = a0.x - b0.y;
            z.y = a0.y + b0.x;
            a[q] = z;
        }
    } else if (active) {
        const C *s0 = spec + ((long)jj * nzp + kk) * nh, *s1 = spec + ((long)jj * nzp + kk + 1) * nh;
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
    C *r = fft_line<N, C>(a, b, pl, tw, tid, G);
    if (!active) return;
    long base0 = (long)n * (jj + (long)nym * kk), base1 = (long)n * (jj + (long)nym * (kk + 1));
#pragma unroll
    for (int q = tid; q < (N > 0 ? N : n); q += (N > 0 ? fft_x_threads(N) : G)) {
        phi[base0 + q] = r[q].x * scale;
        phi[base1 + q] = r[q].y * scale;
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

// reciprocal spacings of the split path's projection
struct RSpG {
    const float *rxg, *ryg, *rzg;  // 1/(xg(i)-xg(i-1)) etc., 1-based
};

// planes per thread of the pressure store: every load of the thread is
// issued before the first store
constexpr int PROJ_KP = 2;

// Everything the projection kernel reads: fields as plain pointers (low
// words null unless the update is compensated), phi, reciprocal spacings
// (split path) or coordinates (FP64 path, 1-based), extents.
template <typename T>
struct ProjArgs {
    T *u, *v, *w, *ul, *vl, *wl;
    const T *phi;
    const float *rxg, *ryg, *rzg;
    const T *xg, *yg, *zg;
    int nx, ny, nz, nxg, nyg, nzg, nxp, nym, nzp, ilim, klim;
};

// planes per thread of the projection kernel
constexpr int PROJ3_KP = 4;

// The periodic image of canonical index i on an axis of extent n (0: none):
// at centres (extent np + 3) images of 2, 3 and np + 1, at faces (extent
// np + 2) images of 2 and np + 1; at most one per cell when np >= 4 (checked
// on the host).
__device__ __forceinline__ int img_of(int i, int n, bool centre) {
    if (centre) return i == 2 ? n - 1 : (i == 3 ? n : (i == n - 2 ? 1 : 0));
    return i == 2 ? n : (i == n - 1 ? 1 : 0);
}

// The ghost copies apply_boundary_conditions (boundary_conditions.f90:20-75)
// makes of a canonical cell (i, j, k) of one field with no-slip walls: its
// periodic images in x and z (update of the duplicate columns and planes,
// :87-244) and, on the rows next to a wall, the wall ghost of the cell and of
// each image (:257-272): -value at y centres, 0 at y faces.  F: the field
// with row stride sy and plane stride sz (1-based indices), extents n1 x n2
// x n3; xc / zc: x / z centres, yf: y faces.
template <typename T, bool LO>
__device__ __forceinline__ void put_images(T *F, T *Fl, int sy, int sz, int n1, int n2, int n3, bool xc, bool zc,
                                           bool yf, int i, int j, int k, T v, T vl) {
    const int xi = img_of(i, n1, xc), zi = img_of(k, n3, zc);
    const bool yw = j == 2 || j == n2 - 1;
    if (!(xi | zi) && !yw) return;
    auto put = [&](int ii, int jj, int kk, T x, T xl) {
        const int o = (ii - 1) + sy * (jj - 1) + sz * (kk - 1);
        F[o] = x;
        if constexpr (LO) Fl[o] = xl;
    };
    if (xi) put(xi, j, k, v, vl);
    if (zi) put(i, j, zi, v, vl);
    if (xi && zi) put(xi, j, zi, v, vl);
    if (yw) {
        const int jg = j == 2 ? 1 : n2;
        const T gv = yf ? T(0) : -v, gl = yf ? T(0) : -vl;
        put(i, jg, k, gv, gl);
        if (xi) put(xi, jg, k, gv, gl);
        if (zi) put(i, jg, zi, gv, gl);
        if (xi && zi) put(xi, jg, zi, gv, gl);
    }
}

// project_velocity (projection.f90:203-225) of the three components, one
// thread per (i, j) column and PROJ3_KP planes; ilim, klim: last x and z
// index projected (nxg-1 and nzg-1 for the full interior; nxp+1 and nzp+1
// for the canonical cells only).  LO: the compensated update of the split
// path's last substep (hi + lo).  IMG (canonical cells, no-slip walls):
// every ghost copy of the new values is written as well, which is what
// apply_boundary_conditions after the projection would do -- by the few
// threads whose cells have any, after the main stores, from the values they
// have just stored.  phi is read through the periodic wrap, which reproduces
// apply_periodic_xz_pressure (projection.f90:144-162).  Every index is formed
// once per thread; planes follow by adding the plane strides.
template <typename T, bool IMG, bool LO>
__global__ void __launch_bounds__(128) k_project3(const __grid_constant__ ProjArgs<T> a) {
    constexpr int KP = PROJ3_KP;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
    const int k0 = blockIdx.z * KP + 2;
    const int nx = a.nx, ny = a.ny, nz = a.nz, nxg = a.nxg, nyg = a.nyg, nzg = a.nzg, klim = a.klim;
    if (i > a.ilim || j > nyg - 1) return;
    const bool du = i <= nx - 1, dv = j <= ny - 1;
    // phi offsets: canonical x of i and i+1, rows j and j+1, planes
    const int nxp = a.nxp, pls = nxp * a.nym;
    const int ic0 = wrapf(i, nxp) - 2 + nxp * (j - 2), ic1 = wrapf(i + 1, nxp) - 2 + nxp * (j - 2), jc1 = ic0 + nxp;
    int kof[KP + 1];
#pragma unroll
    for (int q = 0; q <= KP; q++) kof[q] = pls * (wrapf(k0 + q, a.nzp) - 2);
    // field indices (1-based, the reference's extents) of plane k0
    const int suy = nx, suz = nx * nyg, svy = nxg, svz = nxg * ny, swy = nxg, swz = nxg * nyg;
    const int iu = (i - 1) + suy * (j - 1) + suz * (k0 - 1), iv = (i - 1) + svy * (j - 1) + svz * (k0 - 1),
              iw = (i - 1) + swy * (j - 1) + swz * (k0 - 1);
    const T *__restrict__ phi = a.phi;
    T p0[KP + 1], px[KP], py[KP], u[KP], v[KP], w[KP], ul[KP], vl[KP], wl[KP];
#pragma unroll
    for (int q = 0; q <= KP; q++) p0[q] = k0 + q <= nzg - 1 ? phi[ic0 + kof[q]] : T(0);
#pragma unroll
    for (int q = 0; q < KP; q++) {
        const int k = k0 + q;
        const bool kin = k <= klim, dw = k <= nz - 1;
        px[q] = du && kin ? phi[ic1 + kof[q]] : T(0);
        py[q] = dv && kin ? phi[jc1 + kof[q]] : T(0);
        u[q] = du && kin ? a.u[iu + q * suz] : T(0);
        v[q] = dv && kin ? a.v[iv + q * svz] : T(0);
        w[q] = dw && kin ? a.w[iw + q * swz] : T(0);
        if constexpr (LO) {
            ul[q] = du && kin ? a.ul[iu + q * suz] : T(0);
            vl[q] = dv && kin ? a.vl[iv + q * svz] : T(0);
            wl[q] = dw && kin ? a.wl[iw + q * swz] : T(0);
        }
    }
    T rx, ry;
    if constexpr (sizeof(T) == 4) {
        rx = du ? a.rxg[i + 1] : T(0);
        ry = dv ? a.ryg[j + 1] : T(0);
    } else {
        rx = du ? T(1) / (a.xg[i + 1] - a.xg[i]) : T(0);
        ry = dv ? T(1) / (a.yg[j + 1] - a.yg[j]) : T(0);
    }
    auto upd = [&](T *F, T *Fl, int o, T f, T fl, T gr) {
        if constexpr (sizeof(T) == 4 && LO) {
            float hi = f, l = fl;
            ff_add(hi, l, -gr);
            F[o] = hi;
            Fl[o] = l;
        } else {
            F[o] = f - gr;
        }
    };
#pragma unroll
    for (int q = 0; q < KP; q++) {
        const int k = k0 + q;
        if (k > klim) break;
        T gx, gy, gz;
        if constexpr (sizeof(T) == 4) {
            gx = (px[q] - p0[q]) * rx;
            gy = (py[q] - p0[q]) * ry;
            gz = k <= nz - 1 ? (p0[q + 1] - p0[q]) * a.rzg[k + 1] : T(0);
        } else {
            // projection.f90:209-223 divides by the spacings
            gx = du ? (px[q] - p0[q]) / (a.xg[i + 1] - a.xg[i]) : T(0);
            gy = dv ? (py[q] - p0[q]) / (a.yg[j + 1] - a.yg[j]) : T(0);
            gz = k <= nz - 1 ? (p0[q + 1] - p0[q]) / (a.zg[k + 1] - a.zg[k]) : T(0);
        }
        (void)rx;
        (void)ry;
        if (du) upd(a.u, a.ul, iu + q * suz, u[q], ul[q], gx);
        if (dv) upd(a.v, a.vl, iv + q * svz, v[q], vl[q], gy);
        if (k <= nz - 1) upd(a.w, a.wl, iw + q * swz, w[q], wl[q], gz);
    }
    if constexpr (IMG) {
        const bool ex = i <= 3 || i >= nxg - 2, ey = j == 2 || j >= ny - 1, ez = k0 <= 3 || k0 + KP - 1 >= nzg - 2;
        if (ex || ey || ez) {
#pragma unroll 1
            for (int q = 0; q < KP; q++) {
                const int k = k0 + q;
                if (k > klim) break;
                if (du) {
                    const int o = iu + q * suz;
                    put_images<T, LO>(a.u, a.ul, suy, suz, nx, nyg, nzg, false, true, false, i, j, k, a.u[o],
                                      LO ? a.ul[o] : T(0));
                }
                if (dv) {
                    const int o = iv + q * svz;
                    put_images<T, LO>(a.v, a.vl, svy, svz, nxg, ny, nzg, true, true, true, i, j, k, a.v[o],
                                      LO ? a.vl[o] : T(0));
                }
                if (k <= nz - 1) {
                    const int o = iw + q * swz;
                    put_images<T, LO>(a.w, a.wl, swy, swz, nxg, nyg, nz, true, false, false, i, j, k, a.w[o],
                                      LO ? a.wl[o] : T(0));
                }
            }
        }
    }
}

// P = phi/(dt rk_coef(1,1)) on the full extents, ghosts from the nearest
// interior cell (projection.f90:129-137, 144-162); KP planes per thread.
template <typename T>
__global__ void __launch_bounds__(128) k_store_p(Fld<T> P, const T *__restrict__ phi, PhiView pv, const DevScal *ds,
                                                 T c11, int nxg, int nyg, int nzg) {
    constexpr int KP = PROJ_KP;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k0 = blockIdx.z * KP + 1;
    if (i > nxg || j > nyg) return;
    const int ic = min(max(i, 2), nxg - 1), jc = min(max(j, 2), nyg - 1);
    T v[KP];
#pragma unroll
    for (int q = 0; q < KP; q++) {
        const int kc = min(max(k0 + q, 2), nzg - 1);
        v[q] = k0 + q <= nzg ? phi[pv(ic, jc, kc)] : T(0);
    }
    const T den = ds_dt<T>(ds) * c11;
#pragma unroll
    for (int q = 0; q < KP; q++)
        if (k0 + q <= nzg) P(i, j, k0 + q) = v[q] / den;
}

template <typename T>
static size_t smem_pairs(int n, int LP) {
    return (size_t)LP * 2 * n * sizeof(typename C2<T>::t);
}

// phi = Laplacian^-1 div(U, V, W) on the canonical cells: the forward
// transforms with the divergence fused, the per-mode tridiagonal solves and
// the inverse transforms (projection.f90:40-120), each phase on request (an
// ensemble solves the tridiagonal systems of all its members in one launch).  U, V, W have the extents
// of the velocity fields; only their canonical cells, the x and z neighbours
// below them (read through the periodic wrap) and the wall rows of V are read.
template <typename T>
static int poisson_solve(cf_ctx *ctx, Fld<T> U, Fld<T> V, Fld<T> W, int phases) {
    typedef typename C2<T>::t C;
    GeoT<T> g = geo_of<T>(ctx);
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
    const long npairs = (long)nym * (nzp / 2);
    const long nlines = (long)nym * nh;
    // x transforms: LP line pairs per block, Gx threads per line
    const int Gx = fft_x_threads(nxp);
    int LP = 8;
    while (LP > 1 && smem_pairs<T>(nxp, LP) + nxp * sizeof(C) > 96 * 1024) LP /= 2;
    const size_t shx = smem_pairs<T>(nxp, LP) + nxp * sizeof(C);
    // z transforms: LB lines per block, Gz threads per line
    const int Gz = 16;
    int LB = 16;  // with Gz = 16: FFTZ_KZS elements apart per thread in the copies
    while (LB > 1 && smem_pairs<T>(nzp, LB) + (LB + nzp) * sizeof(C) > 96 * 1024) LB /= 2;
    const size_t shz = smem_pairs<T>(nzp, LB) + (LB + nzp) * sizeof(C);
    RSp rs;
    rs.rx = ctx->d_rgeo_f + ctx->rgeo_off[0];
    rs.ry = ctx->d_rgeo_f + ctx->rgeo_off[2];
    rs.rz = ctx->d_rgeo_f + ctx->rgeo_off[4];
#define CF_FFT_SIZES(X) X(16) X(32) X(64) X(96) X(128) X(192) X(256) X(384) X(512)
#define CF_FWDX(N) case N: \
    if constexpr (xr_r(N, 0) > 0) k_fwd_xr<T, N><<<cdiv(npairs, ZR_T / XR_FT), ZR_T, xr_fwd_smem<T, N>(), ctx->st>>>(g, U, V, W, spec, twxf, rs); \
    else k_fwd_x<T, N><<<cdiv(npairs, LP), LP * Gx, shx, ctx->st>>>(g, U, V, W, spec, px, twxf, LP, rs); \
    break;
#define CF_FFTZ(N, TW) case N: \
    if constexpr (zr_r0(N) > 0) k_fft_zr<T, N><<<cdiv(nlines, ZR_T / zr_threads(N)), ZR_T, zr_smem<T, N>(), ctx->st>>>(spec, TW, (int)nlines, nh); \
    else if constexpr (zr3_r(N, 0) > 0) k_fft_zr3<T, N><<<cdiv(nlines, ZR_T / ZR3_G), ZR_T, zr3_smem<T, N>(), ctx->st>>>(spec, TW, (int)nlines, nh); \
    else k_fft_z<T, N><<<cdiv(nlines, LB), LB * Gz, shz, ctx->st>>>(spec, pz, TW, (int)nlines, nh, LB); \
    break;
#define CF_FFTZF(N) CF_FFTZ(N, twzf)
#define CF_FFTZB(N) CF_FFTZ(N, twzb)
#define CF_INVX(N) case N: \
    if constexpr (xr_r(N, 0) > 0) k_inv_xr<T, N><<<cdiv(npairs, ZR_T / xr_threads(N)), ZR_T, xr_smem<T, N>(), ctx->st>>>(spec, phi, twxb, nym, nzp, scale); \
    else k_inv_x<T, N><<<cdiv(npairs, LP), LP * Gx, shx, ctx->st>>>(spec, phi, px, twxb, nym, nzp, LP, scale); \
    break;
    if (phases & POISSON_FWD) {
    // forward x (divergence fused)
    switch (nxp) {
        CF_FFT_SIZES(CF_FWDX)
        default: k_fwd_x<T, 0><<<cdiv(npairs, LP), LP * Gx, shx, ctx->st>>>(g, U, V, W, spec, px, twxf, LP, rs);
    }
    count_launch(ctx, "k_fwd_x");
    // forward z
    switch (nzp) {
        CF_FFT_SIZES(CF_FFTZF)
        default: k_fft_z<T, 0><<<cdiv(nlines, LB), LB * Gz, shz, ctx->st>>>(spec, pz, twzf, (int)nlines, nh, LB);
    }
    count_launch(ctx, "k_fft_z");
    }
    if (phases & POISSON_TRI) {
    // tridiagonal
    const long NM = (long)nzp * nh;
    TriFac tf;
    size_t nf = (size_t)nym * NM;
    tf.m = ctx->tri_fac;
    tf.rd = ctx->tri_fac + nf;
    tf.du = ctx->tri_fac + 2 * nf;
    tf.dl = ctx->tri_fac + 3 * nf;
    tf.piv = ctx->tri_piv;
    if (sizeof(T) == 4) {
        TriSplit ts;
        ts.l = ctx->tri_l32;
        ts.ru = ctx->tri_ru32;
        ts.du = ctx->tri_du32;
        ts.flag = ctx->tri_flag;
        ts.list = ctx->tri_list;
        ts.nlist = ctx->n_tri_list;
        ts.Dd = ctx->d_tri;
        ts.Dl = ctx->d_tri + nym;
        ts.Du = ctx->d_tri + 2 * nym;
        ts.kxx = ctx->d_tri + 3 * nym;
        ts.kzz = ctx->d_tri + 3 * nym + nxp;
        ts.nh = nh;
        const int rs = tri_split_rs(nym);
        const dim3 tb(32, (nym + rs - 1) / rs);
        const int P = (int)tb.y;
        const size_t per = (tri_refined_smem(nym) + 15) & ~(size_t)15, sb = (size_t)P * 32 * 12;
        const int pw = (int)std::max<size_t>(1, std::min<size_t>(P, TRI_SPLIT_SMEM / per));
        const int npb = cdiv(ts.nlist, pw);
        const size_t sm = std::max(sb, ts.nlist > 0 ? pw * per : 0);
        const unsigned nb = (unsigned)(npb + cdiv(NM, 32));
        if (rs == 16) k_tri_split<16><<<nb, tb, sm, ctx->st>>>((float2 *)spec, tf, ts, nym, NM, npb, pw);
        else k_tri_split<32><<<nb, tb, sm, ctx->st>>>((float2 *)spec, tf, ts, nym, NM, npb, pw);
        count_launch(ctx, "k_tri_split");
    } else {
        k_tri_mode<T><<<(unsigned)NM, 32, tri_mode_smem(nym), ctx->st>>>(spec, tf, nym, NM, nullptr);
        count_launch(ctx, "k_tri_mode");
    }
    }
    if (phases & POISSON_INV) {
    // inverse z
    switch (nzp) {
        CF_FFT_SIZES(CF_FFTZB)
        default: k_fft_z<T, 0><<<cdiv(nlines, LB), LB * Gz, shz, ctx->st>>>(spec, pz, twzb, (int)nlines, nh, LB);
    }
    count_launch(ctx, "k_fft_z");
    // inverse x
    const T scale = T(1.0 / ((double)nxp * (double)nzp));
    switch (nxp) {
        CF_FFT_SIZES(CF_INVX)
        default: k_inv_x<T, 0><<<cdiv(npairs, LP), LP * Gx, shx, ctx->st>>>(spec, phi, px, twxb, nym, nzp, LP, scale);
    }
    count_launch(ctx, "k_inv_x");
    }
#undef CF_FWDX
#undef CF_FFTZ
#undef CF_FFTZF
#undef CF_FFTZB
#undef CF_INVX
    CF_CUDA(cudaGetLastError());
    return 0;
}

template <typename T>
int launch_projection(cf_ctx *ctx, int b, bool store_p, bool lo, bool canon, int phases, bool bc) {
    GeoT<T> g = geo_of<T>(ctx);
    Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    if (int rc = poisson_solve<T>(ctx, U, V, W, phases & POISSON_ALL)) return rc;
    if (!(phases & POISSON_INV)) return 0;  // projection after the inverse transforms
    T *phi = (T *)ctx->phi;
    const int nxp = ctx->nxp, nzp = ctx->nzp, nym = ctx->nym;
    // projection
    PhiView pv;
    pv.nxp = nxp; pv.nym = nym; pv.nzp = nzp;
    dim3 blk(32, 4, 1);
    {
        RSpG rg;
        rg.rxg = ctx->d_rgeo_f + ctx->rgeo_off[1];
        rg.ryg = ctx->d_rgeo_f + ctx->rgeo_off[3];
        rg.rzg = ctx->d_rgeo_f + ctx->rgeo_off[5];
        const int ilim = canon ? ctx->nxp + 1 : ctx->nxg - 1, klim = canon ? ctx->nzp + 1 : ctx->nzg - 1;
        // the boundary conditions as ghost copies written by the projection
        // itself: canonical cells, no-slip walls
        const bool img = bc && canon && ctx->prm.iwall_model == 0 && ctx->nxp >= 4 && ctx->nzp >= 4;
        ProjArgs<T> pa;
        pa.u = (T *)ctx->U[b]; pa.v = (T *)ctx->V[b]; pa.w = (T *)ctx->W[b];
        pa.ul = lo ? (T *)ctx->Ulo[b] : nullptr;
        pa.vl = lo ? (T *)ctx->Vlo[b] : nullptr;
        pa.wl = lo ? (T *)ctx->Wlo[b] : nullptr;
        pa.phi = phi;
        pa.rxg = rg.rxg; pa.ryg = rg.ryg; pa.rzg = rg.rzg;
        pa.xg = g.xg; pa.yg = g.yg; pa.zg = g.zg;
        pa.nx = ctx->nx; pa.ny = ctx->ny; pa.nz = ctx->nz;
        pa.nxg = ctx->nxg; pa.nyg = ctx->nyg; pa.nzg = ctx->nzg;
        pa.nxp = nxp; pa.nym = nym; pa.nzp = nzp;
        pa.ilim = ilim; pa.klim = klim;
        const bool plo = sizeof(T) == 4 && pa.ul != nullptr;
        const dim3 grd(cdiv(ilim - 1, 32), cdiv(ctx->nyg - 2, 4), cdiv(klim - 1, PROJ3_KP));
        if constexpr (sizeof(T) == 4) {
            if (plo) {
                if (img) k_project3<T, true, true><<<grd, blk, 0, ctx->st>>>(pa);
                else k_project3<T, false, true><<<grd, blk, 0, ctx->st>>>(pa);
            }
        }
        if (!plo) {
            if (img) k_project3<T, true, false><<<grd, blk, 0, ctx->st>>>(pa);
            else k_project3<T, false, false><<<grd, blk, 0, ctx->st>>>(pa);
        }
        count_launch(ctx, "k_project3");
        if (img) ctx->state_periodic = true;  // as launch_bc: holds for every later launch on the stream
        else if (bc) {
            if (int rc = launch_bc<T>(ctx, b, lo)) return rc;
        }
    }
    if (store_p) {
        Fld<T> P = make_fld<T>(ctx->P, ctx->nxg, ctx->nyg);
        k_store_p<T><<<dim3(cdiv(ctx->nxg, 32), cdiv(ctx->nyg, 4), cdiv(ctx->nzg, PROJ_KP)), blk, 0, ctx->st>>>(
            P, phi, pv, ctx->ds, 8.0 / 15.0, ctx->nxg, ctx->nyg, ctx->nzg);
        count_launch(ctx, "k_store_p");
    }
    CF_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// Actual pressure, pressure.f90:21-172.
//
// The reference sets the wall rows of rhs_v to bc_1, bc_2 = d/dy(nu dV/dy)
// (pressure.f90:237-247), which puts -bc_1/(y(2)-y(1)) into the divergence
// of row 2 and +bc_2/(y(ny)-y(ny-1)) into row nyg-1, and then adds
// coef_bc_1 (yg(2)-yg(1)) bc_1_hat = bc_1_hat/(y(2)-y(1)) to row 2 and
// subtracts bc_2_hat/(y(ny)-y(ny-1)) from row nyg-1 of every mode
// (pressure.f90:137-139; coef_bc_1 and coef_bc_2 from initialization.f90:
// 357-373).  The transform is linear, so the two contributions cancel
// exactly: the solve below takes zero wall rows in rhs_v and no boundary
// term.  bc_1 and bc_2 then only enter the ghost rows (pressure.f90:158-159).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_zero_vwall(Fld<T> F, int nxg, int ny, int nzg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int k = blockIdx.y + 1;
    if (i > nxg) return;
    F(i, 1, k) = T(0);
    F(i, ny, k) = T(0);
}

// metric factors of the one-sided derivatives at the two walls
// (pressure.f90:283-286, 314-317) and the ghost-row spacings
struct PWall {
    double g[2], g2[2], dyg[2];
};

// d/dy(nu dV/dy) at a wall from V and avg_nu_t (pressure.f90:288-307,
// 319-338); w = 0 bottom, 1 top.  v0..v3: V at the wall and the three faces
// inside, a0 = avg_nu_t at the ghost row, a1 at the first interior row.
__device__ __forceinline__ double wall_dnu_dv(const PWall &pw, int w, double nu, double v0, double v1, double v2,
                                              double v3, double a0, double a1) {
    const double nui = nu + 0.5 * (a0 + a1);
    const double dnu = w == 0 ? (a1 - a0) / pw.dyg[0] : (a0 - a1) / pw.dyg[1];
    const double s = w == 0 ? -1.0 : 1.0;  // the top wall's first derivative runs downwards
    const double dV = (s * 3.0 * v0 - s * 4.0 * v1 + s * v2) / 2.0 / pw.g[w];
    double ddV = 2.0 * v0 - 5.0 * v1 + 4.0 * v2 - 1.0 * v3;
    ddV = (ddV - dV * pw.g2[w]) / (pw.g[w] * pw.g[w]);
    return dnu * dV + nui * ddV;
}

// P on i = 2..nxg-1, j = 1..nyg, k = 2..nzg-1: phi read through the wrap
// (apply_periodic_xz_pressure, pressure.f90:177-195), the wall rows
// P(1) = P(2) - (yg(2)-yg(1)) bc_1 and P(nyg) = P(nyg-1) + (yg(nyg)-yg(nyg-1))
// bc_2 with bc taken at the wrapped column, as the periodic copies that
// follow them in the reference leave it.  The x and z ghost columns are not
// written.
template <typename T>
__global__ void __launch_bounds__(128) k_pressure_store(Fld<T> P, const T *__restrict__ phi, PhiView pv, Fld<T> V,
                                                        const double *__restrict__ avg, PWall pw, double nu, int nxg,
                                                        int ny, int nyg, int nzg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 2;
    if (i > nxg - 1 || j > nyg) return;
    if (j >= 2 && j <= nyg - 1) {
        P(i, j, k) = phi[pv(i, j, k)];
        return;
    }
    const int iw = wrapf(i, pv.nxp), kw = wrapf(k, pv.nzp);
    double bc, pin;
    if (j == 1) {
        bc = wall_dnu_dv(pw, 0, nu, (double)V(iw, 1, kw), (double)V(iw, 2, kw), (double)V(iw, 3, kw),
                         (double)V(iw, 4, kw), avg[1], avg[2]);
        pin = (double)phi[pv(i, 2, k)];
        P(i, j, k) = (T)(pin - pw.dyg[0] * bc);
    } else {
        bc = wall_dnu_dv(pw, 1, nu, (double)V(iw, ny, kw), (double)V(iw, ny - 1, kw), (double)V(iw, ny - 2, kw),
                         (double)V(iw, ny - 3, kw), avg[nyg], avg[nyg - 1]);
        pin = (double)phi[pv(i, nyg - 1, k)];
        P(i, j, k) = (T)(pin + pw.dyg[1] * bc);
    }
}

template <typename T>
int launch_pressure(cf_ctx *ctx, int b) {
    if (ctx->ny < 4) return cf_fail(ctx, CF_ERR_INVALID, "the wall derivatives of the pressure need ny >= 4");
    // right-hand sides of the current fields into slot 1 (pressure.f90:49-51)
    for (int c = 0; c < 3; c++)
        if (int rc = launch_rhs<T>(ctx, c, 0)) return rc;
    Fld<T> Fu = make_fld<T>(ctx->F[0][0], ctx->nx, ctx->nyg);
    Fld<T> Fv = make_fld<T>(ctx->F[0][1], ctx->nxg, ctx->ny);
    Fld<T> Fw = make_fld<T>(ctx->F[0][2], ctx->nxg, ctx->nyg);
    k_zero_vwall<T><<<dim3(cdiv(ctx->nxg, 128), ctx->nzg), 128, 0, ctx->st>>>(Fv, ctx->nxg, ctx->ny, ctx->nzg);
    count_launch(ctx, "k_zero_vwall");
    if (int rc = poisson_solve<T>(ctx, Fu, Fv, Fw, POISSON_ALL)) return rc;
    if (int rc = launch_avg_nu_t_flush(ctx)) return rc;
    const double *y = ctx->hy.data(), *yg = ctx->hyg.data();  // 1-based
    const int ny = ctx->ny, nyg = ctx->nyg;
    PWall pw;
    pw.g[0] = (-3.0 * y[1] + 4.0 * y[2] - y[3]) / 2.0;
    pw.g2[0] = 2.0 * y[1] - 5.0 * y[2] + 4.0 * y[3] - 1.0 * y[4];
    pw.g[1] = (3.0 * y[ny] - 4.0 * y[ny - 1] + y[ny - 2]) / 2.0;
    pw.g2[1] = 2.0 * y[ny] - 5.0 * y[ny - 1] + 4.0 * y[ny - 2] - 1.0 * y[ny - 3];
    pw.dyg[0] = yg[2] - yg[1];
    pw.dyg[1] = yg[nyg] - yg[nyg - 1];
    PhiView pv;
    pv.nxp = ctx->nxp; pv.nym = ctx->nym; pv.nzp = ctx->nzp;
    Fld<T> P = make_fld<T>(ctx->P, ctx->nxg, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    k_pressure_store<T><<<dim3(cdiv(ctx->nxg - 2, 32), cdiv(nyg, 4), ctx->nzg - 2), dim3(32, 4), 0, ctx->st>>>(
        P, (const T *)ctx->phi, pv, V, ctx->avg_nu_t, pw, ctx->prm.nu, ctx->nxg, ny, nyg, ctx->nzg);
    count_launch(ctx, "k_pressure_store");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// smem opt-in for the FFT kernels (called once at context creation)
template <typename T, int N>
static void fft_attrs_one() {
    cudaFuncSetAttribute(k_fwd_x<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_inv_x<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_fft_z<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    if constexpr (zr3_r(N, 0) > 0) {
        cudaFuncSetAttribute(k_fft_zr3<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zr3_smem<T, N>());
        cudaFuncSetAttribute(k_fwd_xr<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xr_fwd_smem<T, N>());
        cudaFuncSetAttribute(k_inv_xr<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xr_smem<T, N>());
    }
    if constexpr (zr_r0(N) > 0) {
        // exactly what the launches request (up to 110 KB: FP64, length 96)
        cudaFuncSetAttribute(k_fft_zr<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zr_smem<T, N>());
        cudaFuncSetAttribute(k_fwd_xr<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xr_fwd_smem<T, N>());
        cudaFuncSetAttribute(k_inv_xr<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xr_smem<T, N>());
    }
}

// smem opt-in for the FFT and tridiagonal kernels (called once at context creation)
int fft_setup_attrs() {
    cudaFuncSetAttribute(k_tri_split<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRI_SPLIT_SMEM);
    cudaFuncSetAttribute(k_tri_split<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRI_SPLIT_SMEM);
#define CF_ATTRS(N) fft_attrs_one<double, N>(); fft_attrs_one<float, N>();
    CF_FFT_SIZES(CF_ATTRS)
    CF_ATTRS(0)
#undef CF_ATTRS
    return 0;
}

template int launch_projection<double>(cf_ctx *, int, bool, bool, bool, int, bool);
template int launch_projection<float>(cf_ctx *, int, bool, bool, bool, int, bool);
template int launch_pressure<double>(cf_ctx *, int);
template int launch_pressure<float>(cf_ctx *, int);
