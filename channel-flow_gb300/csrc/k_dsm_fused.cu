// k_dsm_fused.cu -- the dynamic Smagorinsky pass (subgrid.f90:376-538) as one
// kernel that reads U, V, W once and writes |S| plus the plane partial sums of
// L.M and M.M.
//
// A block owns a TX x TY tile of canonical centres and marches along z over a
// chunk of planes.  Everything the pass needs at an output plane k is built
// from shared-memory rings of three planes:
//   R(p)  raw U, V, W on the tile plus 2 halo cells           (plane p)
//   G(p)  U, V, W filtered in x and y on the tile + 1 halo    (plane p)
//   F(p)  Uf, Vf, Wf = z-filter of G(p-1..p+1)                 (plane p)
//   Q(p)  centre velocities, their products, |S| S_ij and |S| (plane p, one)
// Both x-y filters are separable passes: a column pass per (field or pair,
// column) filters R(p) and Q(p) in y (each column read once for all its
// rows), and each point takes the x filter of three filtered columns.  The
// x-y filtered 15 Q quantities at a thread's own point are spread into
// z-accumulators held in registers (weights 1/6, 2/3, 1/6 to planes p-1, p,
// p+1), so L_ij and hat(|S| S_ij) of plane k are complete once Q(k+1) has
// been filtered; M_ij then needs S_ij of Uf, Vf, Wf at k, i.e. F(k-1..k+1).
// With raw plane r entering the ring, the block therefore emits plane r-2.
// Three barriers per plane: after the raw column pass, after G/F/Q, after
// the Q column pass (with the next raw plane committed and the strain of the
// filtered velocities read before it).
//
// The halo is read through the periodic wrap, which reproduces the
// reference's periodic copies whenever U, V, W are themselves periodic in x
// and z -- true after apply_boundary_conditions with no-slip walls
// (iwall_model 0).  The plane sums count the duplicate column i = nxg-1 and
// plane k = nzg-1 of the reference's loops as weight 2 on i = 2, k = 2.
#include <type_traits>

#include "cf_internal.cuh"

// periodic index for i in [2 - np, 2 np + 1]
__device__ __forceinline__ int wrapq(int i, int np) { return i < 2 ? i + np : (i > np + 1 ? i - np : i); }

// Pairs of quantities filtered together: packed FP32x2 arithmetic (one
// instruction for two lanes of work) in the split path, plain FP64 pairs
// otherwise.
template <typename T> struct PairT;
template <> struct PairT<float> { typedef float2 t; };
template <> struct PairT<double> { typedef double2 t; };

__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 psplat(float a) { return make_float2(a, a); }
__device__ __forceinline__ double2 pfma(double2 a, double2 b, double2 c) {
    return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ double2 pmul(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ double2 psplat(double a) { return make_double2(a, a); }

struct RGeo {  // reciprocal spacings, 1-based like the coordinates
    const void *rdx, *rdxg, *rdy, *rdyg, *rdz, *rdzg;
};

// planes per z chunk at most (their z spacings sit in static shared memory)
constexpr int DSM_ZMAX = DSM_ZMAX_HOST;

template <typename T, int TX, int TY>
struct DsmSmem {
    static constexpr int RX = TX + 4, RY = TY + 4, QX = TX + 2, QY = TY + 2;
    static constexpr int NR = 9 * RX * RY, NG = 9 * QX * QY, NF = 9 * QX * QY, NQ = 16 * QX * QY, NC = 16 * QX * TY,
                         NY = 3 * QY * RX;
    static constexpr size_t bytes = (size_t)(NR + NG + NF + NQ + NC + NY) * sizeof(T);
};

// resident blocks per SM the pass is compiled for (three blocks at 80
// registers spill and run slower than two)
template <typename T> struct DsmMinB { static constexpr int v = 2; };

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(TX *TY, TX * TY >= 512 ? 1 : DsmMinB<T>::v) k_dsm_fused(Fld<T> U, Fld<T> V, Fld<T> W, RGeo rgv, int nx, int ny, int nyg,
                                                      int nz, int nxp, int nzp, int kc_len, T *Sout, double *part,
                                                      int nchunk) {
    typedef DsmSmem<T, TX, TY> SM;
    constexpr int RX = SM::RX, RY = SM::RY, QX = SM::QX, QY = SM::QY;
    extern __shared__ unsigned char sm_raw[];
    T *R = (T *)sm_raw;         // [slot 3][field 3][RY][RX]
    T *G = R + SM::NR;          // [slot 3][field 3][QY][QX]
    T *F = G + SM::NG;          // [slot 3][field 3][QY][QX]
    typedef typename PairT<T>::t PT;
    PT *Qs = (PT *)(F + SM::NF);  // [8 pairs][QY][QX]
    PT *Cs = Qs + SM::NQ / 2;     // [8 pairs][TY][QX]: Q filtered in y
    T *Ry = (T *)(Cs + SM::NC / 2);  // [field 3][QY][RX]: the raw plane filtered in y
    const T *rdx = (const T *)rgv.rdx, *rdxg = (const T *)rgv.rdxg, *rdy = (const T *)rgv.rdy,
            *rdyg = (const T *)rgv.rdyg, *rdz = (const T *)rgv.rdz, *rdzg = (const T *)rgv.rdzg;
    const T f6 = T(1.0 / 6.0), f23 = T(2.0 / 3.0), f13 = T(1.0 / 3.0), h = T(0.5), qq = T(0.25);

    const int i0 = 2 + blockIdx.x * TX, j0 = 2 + blockIdx.y * TY;
    const int kb = 2 + blockIdx.z * kc_len, ke = min(kb + kc_len - 1, nz - 1);
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    const int io = i0 + tx, jo = j0 + ty;
    const bool own = io <= nx - 1 && jo <= nyg - 1;
    auto RS = [&](int slot, int f, int sy, int sx) -> T & { return R[((slot * 3 + f) * RY + sy) * RX + sx]; };
    auto GS = [&](int slot, int f, int sy, int sx) -> T & { return G[((slot * 3 + f) * QY + sy) * QX + sx]; };
    auto FS = [&](int slot, int f, int sy, int sx) -> T & { return F[((slot * 3 + f) * QY + sy) * QX + sx]; };
    auto QS = [&](int p, int sy, int sx) -> PT & { return Qs[(p * QY + sy) * QX + sx]; };
    auto CS = [&](int p, int oy, int sx) -> PT & { return Cs[(p * TY + oy) * QX + sx]; };
    auto YS = [&](int f, int sy, int rx) -> T & { return Ry[(f * QY + sy) * RX + rx]; };

    // y filter weights of a row in [lo, hi] (one-sided at the ends)
    auto yw = [&](int j, int lo, int hi, T &wm, T &w0, T &wp) {
        if (j <= lo) { wm = T(0); w0 = f23; wp = f13; }
        else if (j >= hi) { wm = f13; w0 = f23; wp = T(0); }
        else { wm = f6; w0 = f23; wp = f6; }
    };
    const T fw[3] = {f6, f23, f6};

    // reciprocal spacings of the region columns and rows (z is per plane)
    __shared__ T gsx[3][QX], gsy[3][QY];
    // z spacings of every plane the chunk touches (rs .. re), so that no
    // plane starts with a global load
    __shared__ T gsz[3][DSM_ZMAX + 4];
    {
        const int zs = 2 + blockIdx.z * kc_len - 2, ze = min(2 + blockIdx.z * kc_len + kc_len - 1, nz - 1) + 2;
        for (int t = tid; t <= ze - zs; t += TX * TY) {
            const int kc = wrapc(zs + t, nzp);
            gsz[0][t] = rdz[kc];
            gsz[1][t] = rdzg[kc];
            gsz[2][t] = rdzg[kc + 1];
        }
    }
    for (int t = tid; t < QX; t += TX * TY) {
        int ic = wrapq(i0 + t - 1, nxp);
        gsx[0][t] = rdx[ic];
        gsx[1][t] = rdxg[ic];
        gsx[2][t] = rdxg[ic + 1];
    }
    for (int t = tid; t < QY; t += TX * TY) {
        int jj = min(max(j0 + t - 1, 2), nyg - 1);
        gsy[0][t] = rdy[jj];
        gsy[1][t] = rdyg[jj];
        gsy[2][t] = rdyg[jj + 1];
    }
    // z-accumulators of the x-y filtered pairs (uc,vc) (wc,uu) (vv,ww) (uv,uw)
    // (vw,|S|S11) (|S|S22,|S|S33) (|S|S12,|S|S13) (|S|S23,|S|) for the three
    // planes in flight
    PT acc[3][8];
#pragma unroll
    for (int s = 0; s < 3; s++)
#pragma unroll
        for (int q = 0; q < 8; q++) acc[s][q] = psplat(T(0));
    T Sprev = T(0);
    T sl = T(0), smm = T(0);  // this thread's plane sums (widened per block)

    // this thread's point of the halo ring of the QX x QY region (top row,
    // bottom row, left column, right column), if any
    const bool hal = tid < 2 * QX + 2 * TY;
    int hsx = 0, hsy = 0;
    if (tid < QX) { hsx = tid; hsy = 0; }
    else if (tid < 2 * QX) { hsx = tid - QX; hsy = QY - 1; }
    else if (tid < 2 * QX + TY) { hsx = 0; hsy = tid - 2 * QX + 1; }
    else if (hal) { hsx = QX - 1; hsy = tid - 2 * QX - TY + 1; }
    const int rs = kb - 2, re = ke + 2;
    // one march step for raw plane r; PH = (r - rs) % 3 is the ring phase
    // raw-tile elements of this thread (same for every plane)
    constexpr int NTH = TX * TY, NRP = RX * RY, NLR = (NRP + NTH - 1) / NTH;
    int eia[NLR], eja[NLR], ers[NLR];
#pragma unroll
    for (int q = 0; q < NLR; q++) {
        int rem = tid + q * NTH;
        ers[q] = rem;
        int sy = rem / RX, sx = rem - sy * RX;
        eia[q] = wrapq(i0 + sx - 2, nxp);
        eja[q] = j0 + sy - 2;
    }
    T pre[3][NLR];
    auto fetch = [&](int r) {  // issue every load of raw plane r
        const int kc = wrapn(r, nzp);
#pragma unroll
        for (int q = 0; q < NLR; q++) {
            const bool in = ers[q] < NRP;
            const int ia = eia[q], ja = eja[q];
            pre[0][q] = (in && ja >= 1 && ja <= nyg) ? U(ia, ja, kc) : T(0);
            pre[1][q] = (in && ja >= 1 && ja <= ny) ? V(ia, ja, kc) : T(0);
            pre[2][q] = (in && ja >= 1 && ja <= nyg) ? W(ia, ja, kc) : T(0);
        }
    };
    auto commit = [&](int slot) {
#pragma unroll
        for (int q = 0; q < NLR; q++)
            if (ers[q] < NRP) {
#pragma unroll
                for (int f = 0; f < 3; f++) R[(slot * 3 + f) * NRP + ers[q]] = pre[f][q];
            }
    };
    // one march step for raw plane r; PH = (r - rs) % 3 is the ring phase.
    // On entry R(r) is in slot PH; R(r+1) is fetched during the step.
    auto step = [&](int r, auto PHc) {
        constexpr int PH = decltype(PHc)::value;
        constexpr int P1 = (PH + 1) % 3, P2 = (PH + 2) % 3;
        if (r + 1 <= re) fetch(r + 1);
        // -- y filter of the raw plane R(r) (slot PH), one (field, raw
        // column) per task: the column's RY values give the QY rows of the
        // region (one-sided at rows 1 and jhi); G below is its x filter
        for (int t = tid; t < 3 * RX; t += NTH) {
            const int f = t / RX, rx = t - f * RX, jhi = f == 1 ? ny : nyg;
            T col[RY];
#pragma unroll
            for (int q = 0; q < RY; q++) col[q] = RS(PH, f, q, rx);
#pragma unroll
            for (int sy = 0; sy < QY; sy++) {
                const int j = j0 + sy - 1;
                T wm, w0, wp;
                yw(j, 1, jhi, wm, w0, wp);
                const T cm = j > 1 ? col[sy] : col[sy + 1], cp = j < jhi ? col[sy + 2] : col[sy + 1];
                YS(f, sy, rx) = wm * cm + w0 * col[sy + 1] + wp * cp;
            }
        }
        __syncthreads();
        // G(r), F(r-1) and Q(r-1) at this thread's points of the tile + 1 halo
        // (its own point, and one point of the halo ring for the first
        // 2 QX + 2 TY threads): G and F at a point only need that point's G
        // history, and Q only the raw planes already in the ring.
        const int zq = max(r - 1 - rs, 0);  // plane r-1 (used from r = kb on)
        const T rz = gsz[0][zq], rzg0 = gsz[1][zq], rzg1 = gsz[2][zq];
        for (int pt = 0; pt < 2; pt++) {
            if (pt == 1 && !hal) break;
            const int sx = pt ? hsx : tx + 1, sy = pt ? hsy : ty + 1;
            const int j = j0 + sy - 1;
            // -- G(r): x-y filtered U, V, W
            T gc[3];
#pragma unroll
            for (int f = 0; f < 3; f++) {
                const int jhi = f == 1 ? ny : nyg;
                T g = T(0);
                if (j >= 1 && j <= jhi) {
#pragma unroll
                    for (int a = -1; a <= 1; a++) g += fw[a + 1] * YS(f, sy, sx + 1 + a);
                }
                GS(PH, f, sy, sx) = g;
                gc[f] = g;
            }
            if (r < kb) continue;
            // -- F(r-1) = z filter of G(r-2), G(r-1), G(r)
#pragma unroll
            for (int f = 0; f < 3; f++) FS(P2, f, sy, sx) = f6 * GS(P1, f, sy, sx) + f23 * GS(P2, f, sy, sx) + f6 * gc[f];
            // -- Q(r-1) from R(r-2) [P1], R(r-1) [P2], R(r) [PH]
            if (j < 2 || j > nyg - 1) {
#pragma unroll
                for (int q = 0; q < 8; q++) QS(q, sy, sx) = psplat(T(0));
                continue;
            }
            {
                const int rx = sx + 1, ry = sy + 1;  // raw slot of the centre
                // raw accessors with offsets (di, dj, dk), dk in {-1, 0, 1}
                auto u = [&](int di, int dj, int dk) { return RS(dk < 0 ? P1 : (dk == 0 ? P2 : PH), 0, ry + dj, rx + di); };
                auto v = [&](int di, int dj, int dk) { return RS(dk < 0 ? P1 : (dk == 0 ? P2 : PH), 1, ry + dj, rx + di); };
                auto w = [&](int di, int dj, int dk) { return RS(dk < 0 ? P1 : (dk == 0 ? P2 : PH), 2, ry + dj, rx + di); };
                T uc = h * (u(-1, 0, 0) + u(0, 0, 0));
                T vc = h * (v(0, -1, 0) + v(0, 0, 0));
                T wc = h * (w(0, 0, -1) + w(0, 0, 0));
                // compute_Sij (subgrid.f90:900-946)
                const T rx0 = gsx[0][sx], rxg0 = gsx[1][sx], rxg1 = gsx[2][sx];
                const T ry0 = gsy[0][sy], ryg0 = gsy[1][sy], ryg1 = gsy[2][sy];
                T s0 = (u(0, 0, 0) - u(-1, 0, 0)) * rx0;
                T s1 = (v(0, 0, 0) - v(0, -1, 0)) * ry0;
                T s2 = (w(0, 0, 0) - w(0, 0, -1)) * rz;
                T s3 = T(0), s4 = T(0), s5 = T(0);
#pragma unroll
                for (int a = 0; a < 2; a++)
#pragma unroll
                    for (int b = 0; b < 2; b++) {
                        const T rxa = a ? rxg1 : rxg0, ryb = b ? ryg1 : ryg0, rzb = b ? rzg1 : rzg0, rya = a ? ryg1 : ryg0;
                        s3 += h * ((u(a - 1, b, 0) - u(a - 1, b - 1, 0)) * ryb + (v(a, b - 1, 0) - v(a - 1, b - 1, 0)) * rxa);
                        s4 += h * ((u(a - 1, 0, b) - u(a - 1, 0, b - 1)) * rzb + (w(a, 0, b - 1) - w(a - 1, 0, b - 1)) * rxa);
                        s5 += h * ((v(0, a - 1, b) - v(0, a - 1, b - 1)) * rzb + (w(0, a, b - 1) - w(0, a - 1, b - 1)) * rya);
                    }
                s3 *= qq; s4 *= qq; s5 *= qq;
                T S = sqrt(T(2) * s0 * s0 + T(2) * s1 * s1 + T(2) * s2 * s2 + T(4) * s3 * s3 + T(4) * s4 * s4 +
                           T(4) * s5 * s5);
                PT q0, q1, q2, q3, q4, q5, q6, q7;
                q0.x = uc; q0.y = vc;
                q1.x = wc; q1.y = uc * uc;
                q2.x = vc * vc; q2.y = wc * wc;
                q3.x = uc * vc; q3.y = uc * wc;
                q4.x = vc * wc; q4.y = S * s0;
                q5.x = S * s1; q5.y = S * s2;
                q6.x = S * s3; q6.y = S * s4;
                q7.x = S * s5; q7.y = S;
                QS(0, sy, sx) = q0; QS(1, sy, sx) = q1; QS(2, sy, sx) = q2; QS(3, sy, sx) = q3;
                QS(4, sy, sx) = q4; QS(5, sy, sx) = q5; QS(6, sy, sx) = q6; QS(7, sy, sx) = q7;
            }
        }
        __syncthreads();
        // R(r-2) (slot P1) was last read by Q(r-1): R(r+1) takes its place
        // (visible after the next barrier)
        if (r + 1 <= re) commit(P1);
        // S_ij of Uf, Vf, Wf at the output plane k = r-2 (from F(r-3) [PH],
        // F(r-2) [P1], F(r-1) [P2]) and |S| of Q(r-1) at the own point, read
        // before the barrier: the next step overwrites F(r-3) and Q
        T sf[6], Sf = T(0), Snew = T(0);
#pragma unroll
        for (int q = 0; q < 6; q++) sf[q] = T(0);
        if (r >= kb) {
            // -- y filter of Q(r-1), one (pair, column) of the region per
            // task: the column's QY values are read once and give the TY
            // filtered rows (one-sided at the wall rows j = 2 and nyg-1).
            // Tasks 0 .. 8 TX - 1 take columns 0 .. TX - 1 of one pair per
            // TX lanes; the last 16 take columns TX and TX + 1.
            const bool inner = j0 > 2 && j0 + TY - 1 < nyg - 1;
            for (int t = tid; t < 8 * QX; t += NTH) {
                int q, sx;
                if (t < 8 * TX) { q = t / TX; sx = t - q * TX; }
                else { q = (t - 8 * TX) >> 1; sx = TX + ((t - 8 * TX) & 1); }
                PT col[QY];
#pragma unroll
                for (int s = 0; s < QY; s++) col[s] = QS(q, s, sx);
                if (inner) {
                    const PT pf6 = psplat(f6), pf23 = psplat(f23);
#pragma unroll
                    for (int oy = 0; oy < TY; oy++) {
                        PT c = pmul(pf23, col[oy + 1]);
                        c = pfma(pf6, col[oy], c);
                        c = pfma(pf6, col[oy + 2], c);
                        CS(q, oy, sx) = c;
                    }
                } else {
#pragma unroll
                    for (int oy = 0; oy < TY; oy++) {
                        const int j = j0 + oy;
                        T wm, w0, wp;
                        yw(j, 2, nyg - 1, wm, w0, wp);
                        const PT cm = j > 2 ? col[oy] : col[oy + 1], cp = j < nyg - 1 ? col[oy + 2] : col[oy + 1];
                        PT c = pmul(psplat(w0), col[oy + 1]);
                        c = pfma(psplat(wm), cm, c);
                        c = pfma(psplat(wp), cp, c);
                        CS(q, oy, sx) = c;
                    }
                }
            }
            if (own) {
                const int sx = tx + 1, sy = ty + 1;
                Snew = QS(7, sy, sx).y;
                if (r >= kb + 2) {
                    const int k = r - 2;
                    auto uf = [&](int di, int dj, int dk) { return FS(dk < 0 ? PH : (dk == 0 ? P1 : P2), 0, sy + dj, sx + di); };
                    auto vf = [&](int di, int dj, int dk) { return FS(dk < 0 ? PH : (dk == 0 ? P1 : P2), 1, sy + dj, sx + di); };
                    auto wf = [&](int di, int dj, int dk) { return FS(dk < 0 ? PH : (dk == 0 ? P1 : P2), 2, sy + dj, sx + di); };
                    const T rx0 = gsx[0][sx], rxg0 = gsx[1][sx], rxg1 = gsx[2][sx];
                    const T ry0 = gsy[0][sy], ryg0 = gsy[1][sy], ryg1 = gsy[2][sy];
                    const T rz = gsz[0][k - rs], rzg0 = gsz[1][k - rs], rzg1 = gsz[2][k - rs];
                    T s0 = (uf(0, 0, 0) - uf(-1, 0, 0)) * rx0;
                    T s1 = (vf(0, 0, 0) - vf(0, -1, 0)) * ry0;
                    T s2 = (wf(0, 0, 0) - wf(0, 0, -1)) * rz;
                    T s3 = T(0), s4 = T(0), s5 = T(0);
#pragma unroll
                    for (int a = 0; a < 2; a++)
#pragma unroll
                        for (int b = 0; b < 2; b++) {
                            const T rxa = a ? rxg1 : rxg0, ryb = b ? ryg1 : ryg0, rzb = b ? rzg1 : rzg0, rya = a ? ryg1 : ryg0;
                            s3 += h * ((uf(a - 1, b, 0) - uf(a - 1, b - 1, 0)) * ryb + (vf(a, b - 1, 0) - vf(a - 1, b - 1, 0)) * rxa);
                            s4 += h * ((uf(a - 1, 0, b) - uf(a - 1, 0, b - 1)) * rzb + (wf(a, 0, b - 1) - wf(a - 1, 0, b - 1)) * rxa);
                            s5 += h * ((vf(0, a - 1, b) - vf(0, a - 1, b - 1)) * rzb + (wf(0, a, b - 1) - wf(0, a - 1, b - 1)) * rya);
                        }
                    s3 *= qq; s4 *= qq; s5 *= qq;
                    Sf = sqrt(T(2) * s0 * s0 + T(2) * s1 * s1 + T(2) * s2 * s2 + T(4) * s3 * s3 + T(4) * s4 * s4 +
                              T(4) * s5 * s5);
                    sf[0] = s0; sf[1] = s1; sf[2] = s2; sf[3] = s3; sf[4] = s4; sf[5] = s5;
                }
            }
        }
        __syncthreads();
        // No barrier closes the step: the next step's first writes (G(r+1)
        // over G(r-2), F(r) over F(r-3), Q(r)) touch nothing read below, and
        // the filtered columns are rewritten only after its first barrier.
        if (r >= kb && own) {
            // -- x filter of the y-filtered Q(r-1) at the own point, spread
            // over planes r-2, r-1, r
            const int sx = tx + 1;
            const PT pf6 = psplat(f6), pf23 = psplat(f23);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                PT a = psplat(T(0));
#pragma unroll
                for (int d = -1; d <= 1; d++) a = pfma(psplat(fw[d + 1]), CS(q, ty, sx + d), a);
                acc[P1][q] = pfma(pf6, a, acc[P1][q]);   // plane r-2 (last contribution)
                acc[P2][q] = pfma(pf23, a, acc[P2][q]);  // plane r-1
                acc[PH][q] = pmul(pf6, a);               // plane r (first contribution; the slot held plane r-3)
            }
            if (r >= kb + 2) {
                // -- output plane k = r-2
                const int kcn = wrapn(r - 2, nzp);
                const T fs2 = T(4);  // fil_size**2 (subgrid.f90:156, 463)
                // filtered quantities of plane r-2 in the order uc vc wc uu vv ww uv uw vw |S|S11..|S|S23
                T fq[15];
#pragma unroll
                for (int q = 0; q < 7; q++) {
                    fq[2 * q] = acc[P1][q].x;
                    fq[2 * q + 1] = acc[P1][q].y;
                }
                fq[14] = acc[P1][7].x;
                const T fu = fq[0], fv = fq[1], fwv = fq[2];
                const T pa[6] = {fu, fv, fwv, fu, fu, fv}, pb[6] = {fu, fv, fwv, fv, fwv, fwv};
                T lm = T(0), mm = T(0);
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    T L = fq[3 + q] - pa[q] * pb[q];
                    T M = fs2 * Sf * sf[q] - fq[9 + q];
                    T wq = q < 3 ? T(1) : T(2);
                    lm += wq * L * M;
                    mm += wq * M * M;
                }
                T wgt = (io == 2 ? T(2) : T(1)) * (kcn == 2 ? T(2) : T(1));
                sl += wgt * lm;
                smm += wgt * mm;
                Sout[(long)(io - 2) + (long)nxp * ((jo - 2) + (long)(nyg - 2) * (kcn - 2))] = Sprev;
            }
            Sprev = Snew;  // |S| at plane r-1 for the next output
        }
    };
    fetch(rs);
    commit(0);
    __syncthreads();
    std::integral_constant<int, 0> c0;
    std::integral_constant<int, 1> c1;
    std::integral_constant<int, 2> c2;
    for (int r = rs; r <= re; r += 3) {
        step(r, c0);
        if (r + 1 <= re) step(r + 1, c1);
        if (r + 2 <= re) step(r + 2, c2);
    }
    // plane partials of this block for row jo: reduce over the TX threads of the row
    if constexpr (sizeof(T) == 4 && TX == 32) {
        // one warp per row: a float-float shuffle tree (FP64 instructions are
        // dozens of times the cost of FP32 ones on this part); lane 0 writes
        // (L.M hi, lo, M.M hi, lo)
        float ah = own ? (float)sl : 0.f, al = 0.f, bh = own ? (float)smm : 0.f, bl = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float a1 = __shfl_down_sync(0xffffffffu, ah, o), a2 = __shfl_down_sync(0xffffffffu, al, o);
            const float b1 = __shfl_down_sync(0xffffffffu, bh, o), b2 = __shfl_down_sync(0xffffffffu, bl, o);
            ff_add2(ah, al, a1, a2);
            ff_add2(bh, bl, b1, b2);
        }
        if (tx == 0 && jo <= nyg - 1) {
            const int chunk = blockIdx.x * gridDim.z + blockIdx.z;
            ((float4 *)part)[(long)(jo - 2) * nchunk + chunk] = make_float4(ah, al, bh, bl);
        }
        return;
    }
    __syncthreads();
    double *red = (double *)sm_raw;  // 2 * TX * TY doubles fit in the R ring
    red[2 * tid] = own ? (double)sl : 0.0;
    red[2 * tid + 1] = own ? (double)smm : 0.0;
    __syncthreads();
    if (tx == 0 && jo <= nyg - 1) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < TX; q++) {
            a += red[2 * (ty * TX + q)];
            b += red[2 * (ty * TX + q) + 1];
        }
        int chunk = blockIdx.x * gridDim.z + blockIdx.z;
        part[((long)(jo - 2) * nchunk + chunk) * 2] = a;
        part[((long)(jo - 2) * nchunk + chunk) * 2 + 1] = b;
    }
}

template <typename T>
static void *rgeo_ptr(cf_ctx *ctx) {
    return sizeof(T) == 8 ? (void *)ctx->d_rgeo : (void *)ctx->d_rgeo_f;
}

template <typename T, int TX, int TY>
static int launch_fused_cfg(cf_ctx *ctx, int b, int kc_len) {
    Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    RGeo rg;
    T *base = (T *)rgeo_ptr<T>(ctx);
    rg.rdx = base + ctx->rgeo_off[0];
    rg.rdxg = base + ctx->rgeo_off[1];
    rg.rdy = base + ctx->rgeo_off[2];
    rg.rdyg = base + ctx->rgeo_off[3];
    rg.rdz = base + ctx->rgeo_off[4];
    rg.rdzg = base + ctx->rgeo_off[5];
    int ntx = cdiv(ctx->nxp, TX), nty = cdiv(ctx->nym, TY), nkc = cdiv(ctx->nzp, kc_len);
    int nchunk = ntx * nkc;
    T *S = (T *)ctx->dsm_q + 15 * ctx->nCan;  // |S| slot of the canonical scratch
    size_t sm = DsmSmem<T, TX, TY>::bytes;
    k_dsm_fused<T, TX, TY><<<dim3(ntx, nty, nkc), TX * TY, sm, ctx->st>>>(U, V, W, rg, ctx->nx, ctx->ny, ctx->nyg, ctx->nz,
                                                                        ctx->nxp, ctx->nzp, kc_len, S, ctx->dsm_part,
                                                                        nchunk);
    count_launch(ctx, "k_dsm_fused");
    ctx->dsm_nchunk_fused = nchunk;
    CF_CUDA(cudaGetLastError());
    return 0;
}

// tile shapes: FP32 32 x 8, FP64 16 x 8 (the FP64 kernel needs more registers
// and twice the shared memory per tile).  32 x 16 FP32 tiles (one 512-thread
// block per SM, 144 KB) do less halo work but run about 5 % slower at
// 192 x 128 x 192 cells (fewer blocks to hide each other's barriers); three
// 32 x 8 blocks per SM neither fit in shared memory nor in 80 registers.
template <typename T> struct DsmCfg;
template <> struct DsmCfg<float> { static constexpr int TX = 32, TY = 8; };
template <> struct DsmCfg<double> { static constexpr int TX = 16, TY = 8; };

int dsm_fused_setup() {
    cudaFuncSetAttribute(k_dsm_fused<float, DsmCfg<float>::TX, DsmCfg<float>::TY>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)DsmSmem<float, DsmCfg<float>::TX, DsmCfg<float>::TY>::bytes);
    cudaFuncSetAttribute(k_dsm_fused<double, DsmCfg<double>::TX, DsmCfg<double>::TY>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)DsmSmem<double, DsmCfg<double>::TX, DsmCfg<double>::TY>::bytes);
    return 0;
}

// z-chunk length: about one full wave of resident blocks
template <typename T>
static int plan_t(int nxp, int nym, int nzp, int sms, int *kc, size_t *nchunk) {
    constexpr int TX = DsmCfg<T>::TX, TY = DsmCfg<T>::TY;
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dsm_fused<T, TX, TY>, TX * TY,
                                                  DsmSmem<T, TX, TY>::bytes);
    per_sm = per_sm < 1 ? 1 : per_sm;
    long tiles = (long)cdiv(nxp, TX) * cdiv(nym, TY);
    long nkc = (long)per_sm * sms / (tiles > 0 ? tiles : 1);
    if (nkc < 1) nkc = 1;
    if (nkc > nzp / 8) nkc = nzp / 8 > 0 ? nzp / 8 : 1;
    if (nkc < cdiv(nzp, DSM_ZMAX)) nkc = cdiv(nzp, DSM_ZMAX);
    *kc = cdiv(nzp, nkc);
    *nchunk = (size_t)cdiv(nxp, TX) * cdiv(nzp, *kc);
    return 0;
}

int dsm_fused_plan(int esz, int nxp, int nym, int nzp, int sms, int *kc, size_t *nchunk) {
    return esz == 8 ? plan_t<double>(nxp, nym, nzp, sms, kc, nchunk) : plan_t<float>(nxp, nym, nzp, sms, kc, nchunk);
}

template <typename T>
int launch_dsm_fused(cf_ctx *ctx, int b) {
    return launch_fused_cfg<T, DsmCfg<T>::TX, DsmCfg<T>::TY>(ctx, b, ctx->dsm_kc);
}

template int launch_dsm_fused<double>(cf_ctx *, int);
template int launch_dsm_fused<float>(cf_ctx *, int);
