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
// The march is a two-phase software pipeline with two barriers per raw
// plane r:
//   phase A(r): the raw column tasks store R(r) -- loaded into registers one
//     step earlier, one (field, column) per task -- into the ring and filter
//     it in y from those registers, then issue the loads of R(r+1); the Q
//     column pass filters Q(r-2) in y; the strain rate of Uf, Vf, Wf at the
//     output plane r-3 (from F(r-4), F(r-3), F(r-2)) and |S| of Q(r-2) at the
//     own point go to registers.
//   phase B(r): G(r) (x filter of the y-filtered raw plane), F(r-1) and
//     Q(r-1) at the own and halo points; the x filter of the y-filtered
//     Q(r-2) is added to the z accumulators of planes r-3 (its last
//     contribution), r-2 and r-1 (its first); plane r-3 is output.
// Phase A reads only what phase B of the step before wrote (Q, F) and what it
// writes itself, phase B only what phase A wrote, so one barrier after each
// phase orders every shared-memory access.
//
// The halo is read through the periodic wrap, which reproduces the
// reference's periodic copies whenever U, V, W are themselves periodic in x
// and z -- true after apply_boundary_conditions with no-slip walls
// (iwall_model 0).  With the equilibrium wall model it holds except in the
// wall ghost rows at the seams; the centres that can see those entries (the
// seam band, seam_row / seam_line) are then left to k_dsm_seam.  The plane
// sums count the duplicate column i = nxg-1 and plane k = nzg-1 of the
// reference's loops as weight 2 on i = 2, k = 2.
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

// smallest m >= n with m = 4 (mod 32): the stride of the per-field blocks
// that the raw column tasks store to, so that a warp whose tasks span two
// fields writes disjoint banks (the columns of the second field start 4
// banks after the first field's, past the first field's wrapped columns)
constexpr int bank_pad4(int n) { return n + ((36 - n % 32) % 32); }

template <typename T, int TX, int TY>
struct DsmSmem {
    static constexpr int RX = TX + 4, RY = TY + 4, QX = TX + 2, QY = TY + 2;
    static constexpr int RFS = bank_pad4(RY * RX), YFS = bank_pad4(QY * RX);  // field strides of R and Ry
    static constexpr int NR = 9 * RFS, NG = 9 * QX * QY, NF = 9 * QX * QY, NQ = 16 * QX * QY, NC = 16 * QX * TY,
                         NY = 3 * YFS;
    static constexpr size_t bytes = (size_t)(NR + NG + NF + NQ + NC + NY) * sizeof(T);
};

// resident blocks per SM the pass is compiled for (three blocks at 80
// registers spill and run slower than two)
template <typename T> struct DsmMinB { static constexpr int v = 2; };

// Everything one launch of the pass needs for one channel: the fields of the
// state buffer, the reciprocal spacings, sizes, the z-chunk length and the
// tile grid (ntx x nty x nkc blocks), the |S| output and the plane partials.
template <typename T>
struct DsmArgs {
    Fld<T> U, V, W;
    RGeo rg;
    int nx, ny, nyg, nz, nxp, nzp, kc_len, nchunk, ntx, nty, nkc;
    int seam;  // wall-model state: the centres of seam_centre() are left to k_dsm_seam
    T *Sout;
    double *part;
};

// The tile (bx, by, bz) of one channel: a block of the single-channel launch
// or of the ensemble launch (k_dsm_fused_batch below).
template <typename T, int TX, int TY>
__device__ __forceinline__ void dsm_tile(const DsmArgs<T> &args, int bx, int by, int bz) {
    const Fld<T> U = args.U, V = args.V, W = args.W;
    const RGeo rgv = args.rg;
    const int nx = args.nx, ny = args.ny, nyg = args.nyg, nz = args.nz, nxp = args.nxp, nzp = args.nzp,
              kc_len = args.kc_len, nchunk = args.nchunk;
    T *const Sout = args.Sout;
    double *const part = args.part;
    typedef DsmSmem<T, TX, TY> SM;
    constexpr int RX = SM::RX, RY = SM::RY, QX = SM::QX, QY = SM::QY;
    constexpr int NTH = TX * TY, NRT = 3 * RX;
    // the Q column pass is one (pair, column) task per thread for the TX own
    // columns and 16 tasks for the two halo columns, on threads without a
    // raw column task
    static_assert(TY == 8 && NTH == 8 * TX && NRT + 16 <= NTH, "tile shape of the pipelined DSM pass");
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

    const int i0 = 2 + bx * TX, j0 = 2 + by * TY;
    const int kb = 2 + bz * kc_len, ke = min(kb + kc_len - 1, nz - 1);
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    const int io = i0 + tx, jo = j0 + ty;
    const bool own = io <= nx - 1 && jo <= nyg - 1;
    constexpr int RFS = SM::RFS, YFS = SM::YFS;
    auto RS = [&](int slot, int f, int sy, int sx) -> T & { return R[(slot * 3 + f) * RFS + sy * RX + sx]; };
    auto GS = [&](int slot, int f, int sy, int sx) -> T & { return G[((slot * 3 + f) * QY + sy) * QX + sx]; };
    auto FS = [&](int slot, int f, int sy, int sx) -> T & { return F[((slot * 3 + f) * QY + sy) * QX + sx]; };
    auto QS = [&](int p, int sy, int sx) -> PT & { return Qs[(p * QY + sy) * QX + sx]; };
    auto CS = [&](int p, int oy, int sx) -> PT & { return Cs[(p * TY + oy) * QX + sx]; };
    auto YS = [&](int f, int sy, int rx) -> T & { return Ry[f * YFS + sy * RX + rx]; };
    auto yw = [&](int j, int lo, int hi, T &wm, T &w0, T &wp) {
        if (j <= lo) { wm = T(0); w0 = f23; wp = f13; }
        else if (j >= hi) { wm = f13; w0 = f23; wp = T(0); }
        else { wm = f6; w0 = f23; wp = f6; }
    };
    const T fw[3] = {f6, f23, f6};

    __shared__ T gsx[3][QX], gsy[3][QY];
    __shared__ T gsz[3][DSM_ZMAX + 4];
    {
        const int zs = kb - 2, ze = ke + 2;
        for (int t = tid; t <= ze - zs; t += NTH) {
            const int kc = wrapc(zs + t, nzp);
            gsz[0][t] = rdz[kc];
            gsz[1][t] = rdzg[kc];
            gsz[2][t] = rdzg[kc + 1];
        }
    }
    for (int t = tid; t < QX; t += NTH) {
        int ic = wrapq(i0 + t - 1, nxp);
        gsx[0][t] = rdx[ic];
        gsx[1][t] = rdxg[ic];
        gsx[2][t] = rdxg[ic + 1];
    }
    for (int t = tid; t < QY; t += NTH) {
        int jj = min(max(j0 + t - 1, 2), nyg - 1);
        gsy[0][t] = rdy[jj];
        gsy[1][t] = rdyg[jj];
        gsy[2][t] = rdyg[jj + 1];
    }
    PT acc[3][8];
#pragma unroll
    for (int s = 0; s < 3; s++)
#pragma unroll
        for (int q = 0; q < 8; q++) acc[s][q] = psplat(T(0));
    T S_m2 = T(0), S_m3 = T(0);  // |S| of Q(r-2), Q(r-3) at the own point
    T sl = T(0), smm = T(0);
    // wall-model state: this thread's column and row in the seam band
    // (its output planes in the band are added by k_dsm_seam instead)
    const bool seam_rc = args.seam && seam_row(jo, nyg);
    const bool seam_col = seam_rc && seam_line(io, nxp);

    // halo points of phase B: the first TX points of the rows below and
    // above the tile on one warp each, then the four points past them and
    // the two halo columns (for TX = 32 the accesses of every warp fall in
    // distinct banks)
    const bool hal = tid < 2 * QX + 2 * TY;
    int hsx = 0, hsy = 0;
    if (tid < TX) { hsx = tid; hsy = 0; }
    else if (tid < 2 * TX) { hsx = tid - TX; hsy = QY - 1; }
    else if (tid < 2 * TX + 4) { hsx = TX + (tid & 1); hsy = ((tid - 2 * TX) >> 1) ? QY - 1 : 0; }
    else if (tid < 2 * QX + TY) { hsx = 0; hsy = tid - 2 * QX + 1; }
    else if (hal) { hsx = QX - 1; hsy = tid - 2 * QX - TY + 1; }
    const int rs = kb - 2, re = ke + 2;

    // raw column task: field rf, region column rcx, on the last NRT threads
    // (the halo points of phase B are on the first threads)
    const int rtid = tid - (NTH - NRT);
    const bool has_rt = rtid >= 0;
    const int rf = has_rt ? rtid / RX : 0, rcx = has_rt ? rtid - rf * RX : 0;
    const int ria = wrapq(i0 + rcx - 2, nxp), rjhi = rf == 1 ? ny : nyg;
    const Fld<T> RF = rf == 0 ? U : (rf == 1 ? V : W);
    T colv[RY];
    auto fetch_col = [&](int r) {
        const int kc = wrapn(r, nzp);
#pragma unroll
        for (int q = 0; q < RY; q++) {
            const int j = j0 + q - 2;
            colv[q] = (has_rt && j >= 1 && j <= rjhi) ? RF(ria, j, kc) : T(0);
        }
    };
    // halo-column task of the Q column pass (the 16 threads below the raw
    // column tasks)
    const int htid = tid - (NTH - NRT - 16);
    const bool has_hc = htid >= 0 && htid < 16;
    const int hcq = has_hc ? htid >> 1 : 0, hcx = TX + (htid & 1);
    // the raw plane's y filter has interior weights in every region row
    const bool raw_inner = j0 - 1 > 1 && j0 + TY < rjhi;

    auto colpass = [&](int q, int sx, bool inner) {
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
    };

    auto step = [&](int r, auto PHc) {
        constexpr int PH = decltype(PHc)::value;
        constexpr int P1 = (PH + 1) % 3, P2 = (PH + 2) % 3;
        // ================= phase A(r)
        if (r <= re && has_rt) {
            // R(r): into the ring slot of R(r-3) (last read by Q(r-2) in
            // phase B of the step before), and filtered in y into Ry
#pragma unroll
            for (int q = 0; q < RY; q++) RS(PH, rf, q, rcx) = colv[q];
            if (raw_inner) {
#pragma unroll
                for (int sy = 0; sy < QY; sy++) YS(rf, sy, rcx) = f6 * colv[sy] + f23 * colv[sy + 1] + f6 * colv[sy + 2];
            } else {
#pragma unroll
                for (int sy = 0; sy < QY; sy++) {
                    const int j = j0 + sy - 1;
                    T wm, w0, wp;
                    yw(j, 1, rjhi, wm, w0, wp);
                    const T cm = j > 1 ? colv[sy] : colv[sy + 1], cp = j < rjhi ? colv[sy + 2] : colv[sy + 1];
                    YS(rf, sy, rcx) = wm * cm + w0 * colv[sy + 1] + wp * cp;
                }
            }
            if (r + 1 <= re) fetch_col(r + 1);
        }
        T sf[6], Sf = T(0);
#pragma unroll
        for (int q = 0; q < 6; q++) sf[q] = T(0);
        if (r >= kb + 1) {  // Q(r-2) exists (planes kb-1 .. ke+1)
            const bool inner = j0 > 2 && j0 + TY - 1 < nyg - 1;
            colpass(tid / TX, tx, inner);
            if (has_hc) colpass(hcq, hcx, inner);
            S_m3 = S_m2;
            S_m2 = own ? QS(7, ty + 1, tx + 1).y : T(0);
            if (r >= kb + 3 && own) {
                // S_ij of Uf, Vf, Wf at the output plane k = r-3: F(k-1) [P2],
                // F(k) [PH], F(k+1) [P1]
                const int sx = tx + 1, sy = ty + 1, k = r - 3;
                auto uf = [&](int di, int dj, int dk) { return FS(dk < 0 ? P2 : (dk == 0 ? PH : P1), 0, sy + dj, sx + di); };
                auto vf = [&](int di, int dj, int dk) { return FS(dk < 0 ? P2 : (dk == 0 ? PH : P1), 1, sy + dj, sx + di); };
                auto wf = [&](int di, int dj, int dk) { return FS(dk < 0 ? P2 : (dk == 0 ? PH : P1), 2, sy + dj, sx + di); };
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
        __syncthreads();
        // ================= phase B(r)
        if (r <= re) {
            const int zq = max(r - 1 - rs, 0);  // plane r-1 (used from r = kb on)
            const T rz = gsz[0][zq], rzg0 = gsz[1][zq], rzg1 = gsz[2][zq];
            for (int pt = 0; pt < 2; pt++) {
                if (pt == 1 && !hal) break;
                const int sx = pt ? hsx : tx + 1, sy = pt ? hsy : ty + 1;
                const int j = j0 + sy - 1;
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
#pragma unroll
                for (int f = 0; f < 3; f++) FS(P2, f, sy, sx) = f6 * GS(P1, f, sy, sx) + f23 * GS(P2, f, sy, sx) + f6 * gc[f];
                if (j < 2 || j > nyg - 1) {
#pragma unroll
                    for (int q = 0; q < 8; q++) QS(q, sy, sx) = psplat(T(0));
                    continue;
                }
                const int rx = sx + 1, ry = sy + 1;
                auto u = [&](int di, int dj, int dk) { return RS(dk < 0 ? P1 : (dk == 0 ? P2 : PH), 0, ry + dj, rx + di); };
                auto v = [&](int di, int dj, int dk) { return RS(dk < 0 ? P1 : (dk == 0 ? P2 : PH), 1, ry + dj, rx + di); };
                auto w = [&](int di, int dj, int dk) { return RS(dk < 0 ? P1 : (dk == 0 ? P2 : PH), 2, ry + dj, rx + di); };
                T uc = h * (u(-1, 0, 0) + u(0, 0, 0));
                T vc = h * (v(0, -1, 0) + v(0, 0, 0));
                T wc = h * (w(0, 0, -1) + w(0, 0, 0));
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
        if (r >= kb + 1 && own) {
            // x filter of the y-filtered Q(r-2): planes r-3 (last), r-2, r-1 (first)
            const int sx = tx + 1;
            const PT pf6 = psplat(f6), pf23 = psplat(f23);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                PT a = psplat(T(0));
#pragma unroll
                for (int d = -1; d <= 1; d++) a = pfma(psplat(fw[d + 1]), CS(q, ty, sx + d), a);
                acc[PH][q] = pfma(pf6, a, acc[PH][q]);
                acc[P1][q] = pfma(pf23, a, acc[P1][q]);
                acc[P2][q] = pmul(pf6, a);
            }
            if (r >= kb + 3) {
                const int kcn = wrapn(r - 3, nzp);
                const T fs2 = T(4);  // fil_size**2 (subgrid.f90:156, 463)
                T fq[15];
#pragma unroll
                for (int q = 0; q < 7; q++) {
                    fq[2 * q] = acc[PH][q].x;
                    fq[2 * q + 1] = acc[PH][q].y;
                }
                fq[14] = acc[PH][7].x;
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
                if (!(seam_col || (seam_rc && seam_line(kcn, nzp)))) {
                    sl += wgt * lm;
                    smm += wgt * mm;
                }
                Sout[(long)(io - 2) + (long)nxp * ((jo - 2) + (long)(nyg - 2) * (kcn - 2))] = S_m3;
            }
        }
        __syncthreads();
    };
    fetch_col(rs);
    __syncthreads();
    std::integral_constant<int, 0> c0;
    std::integral_constant<int, 1> c1;
    std::integral_constant<int, 2> c2;
    for (int r = rs; r <= re + 1; r += 3) {
        step(r, c0);
        if (r + 1 <= re + 1) step(r + 1, c1);
        if (r + 2 <= re + 1) step(r + 2, c2);
    }
    if constexpr (sizeof(T) == 4 && TX == 32) {
        float ah = own ? (float)sl : 0.f, al = 0.f, bh = own ? (float)smm : 0.f, bl = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float a1 = __shfl_down_sync(0xffffffffu, ah, o), a2 = __shfl_down_sync(0xffffffffu, al, o);
            const float b1 = __shfl_down_sync(0xffffffffu, bh, o), b2 = __shfl_down_sync(0xffffffffu, bl, o);
            ff_add2(ah, al, a1, a2);
            ff_add2(bh, bl, b1, b2);
        }
        if (tx == 0 && jo <= nyg - 1) {
            const int chunk = bx * args.nkc + bz;
            ((float4 *)part)[(long)(jo - 2) * nchunk + chunk] = make_float4(ah, al, bh, bl);
        }
        return;
    }
    double *red = (double *)sm_raw;
    red[2 * tid] = own ? (double)sl : 0.0;
    red[2 * tid + 1] = own ? (double)smm : 0.0;
    __syncthreads();
    if (tx == 0 && jo <= nyg - 1) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < TX; q++) {
            a += red[2 * (ty * TX + q)];
            b += red[2 * (ty * TX + q) + 1];
        }
        int chunk = bx * args.nkc + bz;
        part[((long)(jo - 2) * nchunk + chunk) * 2] = a;
        part[((long)(jo - 2) * nchunk + chunk) * 2 + 1] = b;
    }
}

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(TX *TY, TX * TY >= 512 ? 1 : DsmMinB<T>::v) k_dsm_fused(DsmArgs<T> a) {
    dsm_tile<T, TX, TY>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One launch over the tiles of several channels (an ensemble): member m owns
// blocks first[m] .. first[m+1]-1, in the order of its own launch's grid.
template <typename T>
struct DsmBatch {
    int n;
    int first[CF_ENS_MAXM + 1];
    DsmArgs<T> a[CF_ENS_MAXM];
};

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(TX *TY, TX * TY >= 512 ? 1 : DsmMinB<T>::v) k_dsm_fused_batch(const __grid_constant__ DsmBatch<T> B) {
    const int bid = blockIdx.x;
    int m = 0;
    while (m + 1 < B.n && bid >= B.first[m + 1]) m++;
    const int l = bid - B.first[m], ntx = B.a[m].ntx, nty = B.a[m].nty;
    dsm_tile<T, TX, TY>(B.a[m], l % ntx, (l / ntx) % nty, l / (ntx * nty));
}

// <LM>/<MM> per row of several channels from their plane partials (the
// single-channel kernels k_dsm_e / k_dsm_e_ff per member block range).
struct DsmEArgs {
    const void *part;
    double *avg;
    int nchunk, nyg, dir, ff;
};
struct DsmEBatch {
    int n;
    int first[CF_ENS_MAXM + 1];
    DsmEArgs a[CF_ENS_MAXM];
};

template <typename T>
static void *rgeo_ptr(cf_ctx *ctx) {
    return sizeof(T) == 8 ? (void *)ctx->d_rgeo : (void *)ctx->d_rgeo_f;
}

template <typename T, int TX, int TY>
static DsmArgs<T> fused_args(cf_ctx *ctx, int b, int kc_len) {
    DsmArgs<T> a;
    a.U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    a.V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    a.W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    T *base = (T *)rgeo_ptr<T>(ctx);
    a.rg.rdx = base + ctx->rgeo_off[0];
    a.rg.rdxg = base + ctx->rgeo_off[1];
    a.rg.rdy = base + ctx->rgeo_off[2];
    a.rg.rdyg = base + ctx->rgeo_off[3];
    a.rg.rdz = base + ctx->rgeo_off[4];
    a.rg.rdzg = base + ctx->rgeo_off[5];
    a.nx = ctx->nx; a.ny = ctx->ny; a.nyg = ctx->nyg; a.nz = ctx->nz; a.nxp = ctx->nxp; a.nzp = ctx->nzp;
    a.kc_len = kc_len;
    a.ntx = cdiv(ctx->nxp, TX);
    a.nty = cdiv(ctx->nym, TY);
    a.nkc = cdiv(ctx->nzp, kc_len);
    a.nchunk = a.ntx * a.nkc;
    a.seam = 0;
    a.Sout = (T *)ctx->dsm_q + 15 * ctx->nCan;  // |S| slot of the canonical scratch
    a.part = ctx->dsm_part;
    return a;
}

template <typename T, int TX, int TY>
static int launch_fused_cfg(cf_ctx *ctx, int b, int kc_len) {
    const DsmArgs<T> a = fused_args<T, TX, TY>(ctx, b, kc_len);
    size_t sm = DsmSmem<T, TX, TY>::bytes;
    k_dsm_fused<T, TX, TY><<<dim3(a.ntx, a.nty, a.nkc), TX * TY, sm, ctx->st>>>(a);
    count_launch(ctx, "k_dsm_fused");
    ctx->dsm_nchunk_fused = ctx->dsm_nchunk_base = a.nchunk;
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
    cudaFuncSetAttribute(k_dsm_fused_batch<float, DsmCfg<float>::TX, DsmCfg<float>::TY>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)DsmSmem<float, DsmCfg<float>::TX, DsmCfg<float>::TY>::bytes);
    cudaFuncSetAttribute(k_dsm_fused_batch<double, DsmCfg<double>::TX, DsmCfg<double>::TY>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)DsmSmem<double, DsmCfg<double>::TX, DsmCfg<double>::TY>::bytes);
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

// ---------------------------------------------------------------------------
// k_dsm_seam: the centres of the seam band (seam_row, seam_line) of the
// wall-model state, computed as the multi-pass route computes them
// (subgrid.f90:376-513 with the periodic fills of :448-458): the quantities
// of stage A at a canonical centre from U, V, W at actual indices, at a
// ghost centre the canonical twin's; Uf, Vf, Wf at a canonical element from
// U, V, W at actual indices (y one-sided at rows 1 and n2), at a ghost
// element the twin's; the 27-point filter of the quantities (y one-sided at
// rows 2 and nyg-1), L, M from S_ij(Uf), L.M and M.M with the plane-sum
// weights.  |S| of the centre is written over the one-pass value.  One warp
// per centre: lanes 0..26 the filter's neighbours, lanes 0..29 the 30
// filtered-velocity elements that S_ij(Uf) reads.  Block (b, row j): its
// warps take the row's band centres in turn and the block's sums go to
// partial slot chunk0 + b of row j (the band's rows only: k_dsm_e and
// k_dsm_e_ff read a row's seam slots only in those rows).
// ---------------------------------------------------------------------------
template <typename T>
struct SeamArgs {
    Fld<T> U, V, W;
    GeoT<T> g;
    RcpT<T> rc;
    int nxp, nzp, nyg, ny;
    int rows[4];                 // the band's rows (blockIdx.y)
    int xs[4], nxs, zs[4], nzs;  // band columns and planes, distinct
    int nchunk, chunk0;          // partial-slot stride and the first seam slot
    T *Sout;
    double *part;
};

// 27 values of one field around a centre (ci, cj, ck), as an accessor
template <typename T>
struct CubeAcc {
    const T *c;
    int ci, cj, ck;
    __device__ __forceinline__ T operator()(int i, int j, int k) const {
        return c[(i - ci + 1) + 3 * (j - cj + 1) + 9 * (k - ck + 1)];
    }
};

// stage C at element (i, j, k) of a field with n2 rows (k_dsm_c_t's order:
// y inside x per plane, then z); a ghost or duplicate element takes the
// canonical twin's value
template <typename T>
__device__ T seam_filt_elem(const Fld<T> &F, int n2, int nxp, int nzp, int i, int j, int k) {
    i = wrapc(i, nxp);
    k = wrapc(k, nzp);
    const T f6 = T(1.0 / 6.0), f23 = T(2.0 / 3.0), f13 = T(1.0 / 3.0);
    T wm, w0, wp;
    if (j == 1) { wm = T(0); w0 = f23; wp = f13; }
    else if (j == n2) { wm = f13; w0 = f23; wp = T(0); }
    else { wm = f6; w0 = f23; wp = f6; }
    const int jm = max(j - 1, 1), jp = min(j + 1, n2);  // weight 0 where clamped
    T gz[3];
#pragma unroll
    for (int dk = -1; dk <= 1; dk++) {
        T g = T(0);
#pragma unroll
        for (int a = -1; a <= 1; a++) {
            const T fa = a == 0 ? f23 : f6;
            g += fa * (wm * F(i + a, jm, k + dk) + w0 * F(i + a, j, k + dk) + wp * F(i + a, jp, k + dk));
        }
        gz[dk + 1] = g;
    }
    return f6 * gz[0] + f23 * gz[1] + f6 * gz[2];
}

template <typename T>
__global__ void __launch_bounds__(256) k_dsm_seam(const __grid_constant__ SeamArgs<T> a) {
    const int j = a.rows[blockIdx.y], nyg = a.nyg, nxp = a.nxp, nzp = a.nzp;
    const long slot = ((long)(j - 2) * a.nchunk + a.chunk0 + blockIdx.x);
    __shared__ double red[8][2];
    __shared__ T cube[8][3][27];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    auto put = [&](double lm, double mm) {
        if constexpr (sizeof(T) == 4) {
            const float lh = (float)lm, mh = (float)mm;
            ((float4 *)a.part)[slot] = make_float4(lh, (float)(lm - (double)lh), mh, (float)(mm - (double)mh));
        } else {
            a.part[slot * 2] = lm;
            a.part[slot * 2 + 1] = mm;
        }
    };
    const T f6 = T(1.0 / 6.0), f23 = T(2.0 / 3.0), f13 = T(1.0 / 3.0), h = T(0.5);
    const T fw[3] = {f6, f23, f6};
    // this lane's filter neighbour and its weight (y one-sided at rows 2 and nyg-1)
    const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
    T wy = dy == 0 ? f23 : f6;
    if (j == 2) wy = dy < 0 ? T(0) : (dy > 0 ? f13 : f23);
    else if (j == nyg - 1) wy = dy > 0 ? T(0) : (dy < 0 ? f13 : f23);
    const T wq = lane < 27 ? fw[dx + 1] * wy * fw[dz + 1] : T(0);
    // this lane's filtered-velocity element (field ef, offsets ex, ey, ez)
    int ef = 0, ex = 0, ey = 0, ez = 0;
    if (lane < 10) {
        ef = 0; ex = (lane & 1) - 1;
        const int m = lane >> 1;
        ey = m < 3 ? m - 1 : 0;
        ez = m < 3 ? 0 : (m == 3 ? -1 : 1);
    } else if (lane < 20) {
        const int l = lane - 10;
        ef = 1;
        if (l < 6) { ex = l % 3 - 1; ey = l / 3 - 1; ez = 0; }
        else { const int m = l - 6; ex = 0; ey = (m & 1) - 1; ez = (m >> 1) ? 1 : -1; }
    } else if (lane < 30) {
        const int l = lane - 20;
        ef = 2;
        if (l < 6) { ex = l % 3 - 1; ey = 0; ez = l / 3 - 1; }
        else { const int m = l - 6; ex = 0; ey = (m & 1) ? 1 : -1; ez = (m >> 1) - 1; }
    }
    const int nxr = max(0, nxp - 4);  // columns 4..nxp-1 (outside the band's columns)
    const long npts = (long)a.nxs * nzp + (long)a.nzs * nxr;
    double slm = 0.0, smm = 0.0;
    for (long p = (long)blockIdx.x * 8 + w; p < npts; p += (long)gridDim.x * 8) {
        int i, k;
        if (p < (long)a.nxs * nzp) {
            i = a.xs[p / nzp];
            k = 2 + (int)(p % nzp);
        } else {
            const long q = p - (long)a.nxs * nzp;
            k = a.zs[q / nxr];
            i = 4 + (int)(q % nxr);
        }
        // the stage-A quantities of this lane's neighbour, weighted
        T qv[16];
#pragma unroll
        for (int c = 0; c < 16; c++) qv[c] = T(0);
        if (wq != T(0)) {
            const int ci = wrapc(i + dx, nxp), cj = j + dy, ck = wrapc(k + dz, nzp);
            const T uc = h * (a.U(ci - 1, cj, ck) + a.U(ci, cj, ck));
            const T vc = h * (a.V(ci, cj - 1, ck) + a.V(ci, cj, ck));
            const T wc = h * (a.W(ci, cj, ck - 1) + a.W(ci, cj, ck));
            T sq[6], S;
            sij_point<T>(a.g, a.rc, a.U, a.V, a.W, ci, cj, ck, sq, S);
            const T qa[15] = {uc, vc, wc, uc * uc, vc * vc, wc * wc, uc * vc, uc * wc, vc * wc,
                              S * sq[0], S * sq[1], S * sq[2], S * sq[3], S * sq[4], S * sq[5]};
#pragma unroll
            for (int c = 0; c < 15; c++) qv[c] = wq * qa[c];
            qv[15] = S;
        }
        // |S| of the centre (lane 13: no offset)
        const T Sc = __shfl_sync(0xffffffffu, qv[15], 13);
        if (lane == 13) a.Sout[(long)(i - 2) + (long)nxp * ((j - 2) + (long)(nyg - 2) * (k - 2))] = Sc;
#pragma unroll
        for (int c = 0; c < 15; c++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) qv[c] += __shfl_xor_sync(0xffffffffu, qv[c], o);
        // the filtered velocities S_ij(Uf) reads
        if (lane < 30) {
            const Fld<T> &F = ef == 0 ? a.U : (ef == 1 ? a.V : a.W);
            cube[w][ef][(ex + 1) + 3 * (ey + 1) + 9 * (ez + 1)] =
                seam_filt_elem<T>(F, ef == 1 ? a.ny : nyg, nxp, nzp, i + ex, j + ey, k + ez);
        }
        __syncwarp();
        if (lane == 0) {
            CubeAcc<T> cu{cube[w][0], i, j, k}, cv{cube[w][1], i, j, k}, cw{cube[w][2], i, j, k};
            T sf[6], Sf;
            sij_point_a<T, CubeAcc<T>>(a.g, a.rc, cu, cv, cw, i, j, k, sf, Sf);
            const T fu = qv[0], fv = qv[1], fwv = qv[2];
            const T pa[6] = {fu, fv, fwv, fu, fu, fv}, pb[6] = {fu, fv, fwv, fv, fwv, fwv};
            T L[6], M[6];
#pragma unroll
            for (int c = 0; c < 6; c++) {
                L[c] = qv[3 + c] - pa[c] * pb[c];
                M[c] = T(4) * Sf * sf[c] - qv[9 + c];  // fil_size**2 = 4 (subgrid.f90:156, 463)
            }
            const T lm = L[0] * M[0] + L[1] * M[1] + L[2] * M[2] + T(2) * (L[3] * M[3] + L[4] * M[4] + L[5] * M[5]);
            const T mm = M[0] * M[0] + M[1] * M[1] + M[2] * M[2] + T(2) * (M[3] * M[3] + M[4] * M[4] + M[5] * M[5]);
            const double wgt = (i == 2 ? 2.0 : 1.0) * (k == 2 ? 2.0 : 1.0);
            slm += wgt * (double)lm;
            smm += wgt * (double)mm;
        }
        __syncwarp();
    }
    if (lane == 0) {
        red[w][0] = slm;
        red[w][1] = smm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int q = 0; q < 8; q++) {
            s0 += red[q][0];
            s1 += red[q][1];
        }
        put(s0, s1);
    }
}

// partial slots per row the seam kernel takes (after the one-pass kernel's):
// a block of 8 warps per 16 band centres of a row (two per warp)
static int seam_slots(int nxp, int nzp) {
    const long npts = 4L * nzp + 4L * std::max(0, nxp - 4);
    return std::max(1, std::min(256, cdiv(npts, 16)));
}
int dsm_seam_slots_max() { return 256; }

template <typename T>
static int launch_seam(cf_ctx *ctx, int b, int chunk0, int nchunk) {
    SeamArgs<T> a;
    a.U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    a.V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    a.W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    a.g = geo_of<T>(ctx);
    a.rc = rcp_of<T>(ctx);
    a.nxp = ctx->nxp; a.nzp = ctx->nzp; a.nyg = ctx->nyg; a.ny = ctx->ny;
    auto band = [](int np, int *out) {
        int n = 0;
        const int c[4] = {2, 3, np, np + 1};
        for (int q = 0; q < 4; q++) {
            bool dup = c[q] < 2 || c[q] > np + 1;
            for (int r = 0; r < n; r++) dup = dup || out[r] == c[q];
            if (!dup) out[n++] = c[q];
        }
        return n;
    };
    a.nxs = band(ctx->nxp, a.xs);
    a.nzs = band(ctx->nzp, a.zs);
    a.nchunk = nchunk;
    a.chunk0 = chunk0;
    a.Sout = (T *)ctx->dsm_q + 15 * ctx->nCan;
    a.part = ctx->dsm_part;
    int nr = 0;
    for (int j : {2, 3, ctx->nyg - 2, ctx->nyg - 1}) {
        bool dup = j < 2 || j > ctx->nyg - 1;
        for (int r = 0; r < nr; r++) dup = dup || a.rows[r] == j;
        if (!dup) a.rows[nr++] = j;
    }
    const int ns = nchunk - chunk0;
    k_dsm_seam<T><<<dim3(ns, nr), 256, 0, ctx->st>>>(a);
    count_launch(ctx, "k_dsm_seam");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// The one-pass kernel on a wall-model state (ghosts filled by the boundary
// conditions): the seam band left to k_dsm_seam, whose partial slots follow
// the one-pass kernel's in every row.
template <typename T>
int launch_dsm_fused_wm(cf_ctx *ctx, int b) {
    constexpr int TX = DsmCfg<T>::TX, TY = DsmCfg<T>::TY;
    DsmArgs<T> a = fused_args<T, TX, TY>(ctx, b, ctx->dsm_kc);
    const int chunk0 = a.nchunk, ns = seam_slots(ctx->nxp, ctx->nzp);
    if ((size_t)(chunk0 + ns) > ctx->dsm_part_nch) return cf_fail(ctx, CF_ERR_INVALID, "plane-partial slots");
    a.nchunk = chunk0 + ns;
    a.seam = 1;
    ctx->dsm_nchunk_base = chunk0;
    size_t sm = DsmSmem<T, TX, TY>::bytes;
    k_dsm_fused<T, TX, TY><<<dim3(a.ntx, a.nty, a.nkc), TX * TY, sm, ctx->st>>>(a);
    count_launch(ctx, "k_dsm_fused");
    CF_CUDA(cudaGetLastError());
    ctx->dsm_nchunk_fused = a.nchunk;
    return launch_seam<T>(ctx, b, chunk0, a.nchunk);
}

template int launch_dsm_fused_wm<double>(cf_ctx *, int);
template int launch_dsm_fused_wm<float>(cf_ctx *, int);

__global__ void __launch_bounds__(256) k_dsm_e_batch(const __grid_constant__ DsmEBatch B) {
    const int bid = blockIdx.x;
    int m = 0;
    while (m + 1 < B.n && bid >= B.first[m + 1]) m++;
    const DsmEArgs &a = B.a[m];
    const int l = bid - B.first[m];
    const int lane = threadIdx.x & 31, j = l * (blockDim.x >> 5) + (threadIdx.x >> 5) + 2, nyg = a.nyg;
    if (j > nyg - 1) return;
    double c;
    if (a.ff) {  // float-float partials (split path), as k_dsm_e_ff
        const float4 *part = (const float4 *)a.part;
        float ah = 0.f, al = 0.f, bh = 0.f, bl = 0.f;
        for (int q = lane; q < a.nchunk; q += 32) {
            const float4 v = part[(long)(j - 2) * a.nchunk + q];
            ff_add2(ah, al, v.x, v.y);
            ff_add2(bh, bl, v.z, v.w);
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float a1 = __shfl_down_sync(0xffffffffu, ah, o), a2 = __shfl_down_sync(0xffffffffu, al, o);
            const float b1 = __shfl_down_sync(0xffffffffu, bh, o), b2 = __shfl_down_sync(0xffffffffu, bl, o);
            ff_add2(ah, al, a1, a2);
            ff_add2(bh, bl, b1, b2);
        }
        c = ((double)ah + (double)al) / ((double)bh + (double)bl);
    } else {  // FP64 partials, as k_dsm_e
        const double *part = (const double *)a.part;
        double s0 = 0.0, s1 = 0.0;
        for (int q = lane; q < a.nchunk; q += 32) {
            s0 += part[((long)(j - 2) * a.nchunk + q) * 2];
            s1 += part[((long)(j - 2) * a.nchunk + q) * 2 + 1];
        }
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_down_sync(0xffffffffu, s0, o);
            s1 += __shfl_down_sync(0xffffffffu, s1, o);
        }
        c = s0 / s1;
    }
    if (lane == 0) {
        double *avg = a.avg;
        float *af = (float *)(avg + nyg + 2);  // FP32 copy for the split path
        avg[j] = c;
        af[j] = (float)c;
        if (j == 2) {
            avg[1] = a.dir ? -c : c;
            af[1] = (float)avg[1];
        }
        if (j == nyg - 1) {
            avg[nyg] = a.dir ? -c : c;
            af[nyg] = (float)avg[nyg];
        }
    }
}

// The one-pass dynamic Smagorinsky pass of n channels (state buffers buf[q])
// in one launch, then their <LM>/<MM> rows in one more: per channel exactly
// the arithmetic of launch_dsm's fused route.  Counts as two launches.
template <typename T>
int launch_dsm_batch(cudaStream_t st, cf_ctx *const *m, const int *buf, int n) {
    constexpr int TX = DsmCfg<T>::TX, TY = DsmCfg<T>::TY;
    if (n < 1 || n > CF_ENS_MAXM) return CF_ERR_INVALID;
    DsmBatch<T> B;
    DsmEBatch E;
    B.n = E.n = n;
    B.first[0] = E.first[0] = 0;
    for (int q = 0; q < n; q++) {
        cf_ctx *c = m[q];
        B.a[q] = fused_args<T, TX, TY>(c, buf[q], c->dsm_kc);
        B.first[q + 1] = B.first[q] + B.a[q].ntx * B.a[q].nty * B.a[q].nkc;
        c->dsm_nchunk_fused = c->dsm_nchunk_base = B.a[q].nchunk;
        E.a[q].part = c->dsm_part;
        E.a[q].avg = c->avg_nu_t;
        E.a[q].nchunk = B.a[q].nchunk;
        E.a[q].nyg = c->nyg;
        E.a[q].dir = c->prm.Dirichlet_nu_t == 1;
        E.a[q].ff = sizeof(T) == 4;
        E.first[q + 1] = E.first[q] + cdiv(c->nym, 8);
        c->nut_lazy = true;
    }
    k_dsm_fused_batch<T, TX, TY><<<B.first[n], TX * TY, DsmSmem<T, TX, TY>::bytes, st>>>(B);
    k_dsm_e_batch<<<E.first[n], 256, 0, st>>>(E);
    return cudaGetLastError() == cudaSuccess ? 0 : CF_ERR_CUDA;
}

template int launch_dsm_batch<double>(cudaStream_t, cf_ctx *const *, const int *, int);
template int launch_dsm_batch<float>(cudaStream_t, cf_ctx *const *, const int *, int);
