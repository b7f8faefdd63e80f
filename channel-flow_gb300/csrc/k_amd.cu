// k_amd.cu -- anisotropic minimum dissipation eddy viscosity,
// subgrid.f90:639-881, in one pass.
//
// The reference builds the model from whole-array and array-section
// operations on the temporaries term, term_1..term_4 (squared or plain
// velocity differences, each moved to the cell centre by two or three
// interpolate_x/_y/_z calls of interpolation.f90:24-105).  At a canonical
// centre (i = 2..nx-1, j = 2..nyg-1, k = 2..nz-1) every one of those
// operations reduces to 27 differences of U, V, W in the cell's 3x3x3
// neighbourhood, combined with weights 1/2; the kernel evaluates that
// reduced form per cell in the order the reference accumulates it.  The
// values the reference computes outside the canonical cells are all
// overwritten by its periodic copies and the wall rule (subgrid.f90:873-876),
// so each canonical value is also written to the duplicate and ghost
// positions that copy it.
//
// A block owns a TX x TY tile of (i, j) columns and marches along z over a
// chunk of planes with planes k-1, k, k+1 of U, V, W (tile plus one halo
// cell) in a shared-memory ring, like the fused right-hand side.
#include "cf_internal.cuh"

namespace {

constexpr int AMD_TX = 32, AMD_TY = 8;

template <typename T>
struct AmdRing {
    static constexpr int SX = AMD_TX + 2;
    const T *b[3];  // planes k-1, k, k+1
    int i0, j0, kc;
    __device__ __forceinline__ T operator()(int i, int j, int k) const {
        return b[k - kc + 1][(j - j0 + 1) * SX + (i - i0 + 1)];
    }
};

// spacing quotients: a / (c(e) - c(e-1)) and a / (c(e) - c(e-1))^2, divided
// as the reference does in FP64, multiplied by the stored reciprocal in FP32
template <typename T>
struct Sp {
    const T *c, *r;
    __device__ __forceinline__ T q1(T a, int e) const {
        if constexpr (sizeof(T) == 8) return a / (c[e] - c[e - 1]);
        else return a * r[e];
    }
    __device__ __forceinline__ T q2(T a, int e) const {
        if constexpr (sizeof(T) == 8) {
            const T d = c[e] - c[e - 1];
            return a / (d * d);
        } else {
            const T q = r[e];
            return a * (q * q);
        }
    }
};

// -C num/den at one canonical centre (subgrid.f90:658-868), clipped with
// NaN -> 0 (subgrid.f90:871).  Differences, with a, b, c in {0, 1}:
//   ux = U(i)-U(i-1);  uy[a][b] = U(i+a-1, j+b) - U(i+a-1, j+b-1);
//   uz[a][c] = U(i+a-1, k+c) - U(i+a-1, k+c-1);  vy = V(j)-V(j-1);
//   vx[a][b] = V(i+a, j+b-1) - V(i+a-1, j+b-1);  vz[b][c] = V(j+b-1, k+c) - V(j+b-1, k+c-1);
//   wz = W(k)-W(k-1);  wx[a][c] = W(i+a, k+c-1) - W(i+a-1, k+c-1);
//   wy[b][c] = W(j+b, k+c-1) - W(j+b-1, k+c-1).
// compute_Sij (subgrid.f90:891-949) takes its edge values from the same
// differences.
template <typename T, typename A>
__device__ __forceinline__ T amd_point(const Sp<T> &sx, const Sp<T> &sxg, const Sp<T> &sy, const Sp<T> &syg,
                                       const Sp<T> &sz, const Sp<T> &szg, const A &U, const A &V, const A &W, int i,
                                       int j, int k) {
    const T h = T(0.5), q = T(0.25), two = T(2);
    const T ux = U(i, j, k) - U(i - 1, j, k);
    const T vy = V(i, j, k) - V(i, j - 1, k);
    const T wz = W(i, j, k) - W(i, j, k - 1);
    T uy[2][2], uz[2][2], vx[2][2], vz[2][2], wx[2][2], wy[2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
            uy[a][b] = U(i + a - 1, j + b, k) - U(i + a - 1, j + b - 1, k);
            uz[a][b] = U(i + a - 1, j, k + b) - U(i + a - 1, j, k + b - 1);
            vx[a][b] = V(i + a, j + b - 1, k) - V(i + a - 1, j + b - 1, k);
            vz[a][b] = V(i, j + a - 1, k + b) - V(i, j + a - 1, k + b - 1);
            wx[a][b] = W(i + a, j, k + b - 1) - W(i + a - 1, j, k + b - 1);
            wy[a][b] = W(i, j + a, k + b - 1) - W(i, j + a - 1, k + b - 1);
        }
    auto av = [h](T p, T r) { return h * (p + r); };
    // Sij at the centre
    const T s11 = sx.q1(ux, i), s22 = sy.q1(vy, j), s33 = sz.q1(wz, k);
    T e4[2][2], e5[2][2], e6[2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
            e4[a][b] = h * (syg.q1(uy[a][b], j + b) + sxg.q1(vx[a][b], i + a));
            e5[a][b] = h * (szg.q1(uz[a][b], k + b) + sxg.q1(wx[a][b], i + a));
            e6[a][b] = h * (szg.q1(vz[a][b], k + b) + syg.q1(wy[a][b], j + a));
        }
    const T s12 = q * (e4[0][0] + e4[1][0] + e4[0][1] + e4[1][1]);
    const T s13 = q * (e5[0][0] + e5[1][0] + e5[0][1] + e5[1][1]);
    const T s23 = q * (e6[0][0] + e6[1][0] + e6[0][1] + e6[1][1]);

    // (d_i u_j)(d_i u_j): term_4 (subgrid.f90:662-763)
    T den = sx.q2(ux * ux, i);
    den = den + av(av(syg.q2(uy[0][0] * uy[0][0], j), syg.q2(uy[1][0] * uy[1][0], j)),
                   av(syg.q2(uy[0][1] * uy[0][1], j + 1), syg.q2(uy[1][1] * uy[1][1], j + 1)));
    den = den + av(av(szg.q2(uz[0][0] * uz[0][0], k), szg.q2(uz[1][0] * uz[1][0], k)),
                   av(szg.q2(uz[0][1] * uz[0][1], k + 1), szg.q2(uz[1][1] * uz[1][1], k + 1)));
    den = den + sy.q2(vy * vy, j);
    den = den + av(av(sxg.q2(vx[0][0] * vx[0][0], i), sxg.q2(vx[0][1] * vx[0][1], i)),
                   av(sxg.q2(vx[1][0] * vx[1][0], i + 1), sxg.q2(vx[1][1] * vx[1][1], i + 1)));
    den = den + av(av(szg.q2(vz[0][0] * vz[0][0], k), szg.q2(vz[1][0] * vz[1][0], k)),
                   av(szg.q2(vz[0][1] * vz[0][1], k + 1), szg.q2(vz[1][1] * vz[1][1], k + 1)));
    den = den + sz.q2(wz * wz, k);
    den = den + av(av(sxg.q2(wx[0][0] * wx[0][0], i), sxg.q2(wx[0][1] * wx[0][1], i)),
                   av(sxg.q2(wx[1][0] * wx[1][0], i + 1), sxg.q2(wx[1][1] * wx[1][1], i + 1)));
    den = den + av(av(syg.q2(wy[0][0] * wy[0][0], j), syg.q2(wy[0][1] * wy[0][1], j)),
                   av(syg.q2(wy[1][0] * wy[1][0], j + 1), syg.q2(wy[1][1] * wy[1][1], j + 1)));

    // (d_hat_k u_i)(d_hat_k u_j) S_ij: nu_t_ (subgrid.f90:660-866)
    auto s2 = [](T p) { return p * p; };
    T num = s2(ux) * s11;
    num = num + av(av(s2(uy[0][0]), s2(uy[1][0])), av(s2(uy[0][1]), s2(uy[1][1]))) * s11;
    num = num + av(av(s2(uz[0][0]), s2(uz[1][0])), av(s2(uz[0][1]), s2(uz[1][1]))) * s11;
    num = num + s2(vy) * s22;
    num = num + av(av(s2(vx[0][0]), s2(vx[0][1])), av(s2(vx[1][0]), s2(vx[1][1]))) * s22;
    num = num + av(av(s2(vz[0][0]), s2(vz[1][0])), av(s2(vz[0][1]), s2(vz[1][1]))) * s22;
    num = num + s2(wz) * s33;
    num = num + av(av(s2(wx[0][0]), s2(wx[0][1])), av(s2(wx[1][0]), s2(wx[1][1]))) * s33;
    num = num + av(av(s2(wy[0][0]), s2(wy[0][1])), av(s2(wy[1][0]), s2(wy[1][1]))) * s33;
    // S12 (subgrid.f90:769-800)
    num = num + two * (av(av(vx[0][0], vx[0][1]), av(vx[1][0], vx[1][1])) * ux) * s12;
    num = num + two * (av(av(uy[0][0], uy[1][0]), av(uy[0][1], uy[1][1])) * vy) * s12;
    num = num + two * av(av(uz[0][0], uz[1][0]) * av(vz[0][0], vz[1][0]), av(uz[0][1], uz[1][1]) * av(vz[0][1], vz[1][1])) * s12;
    // S13 (subgrid.f90:802-833)
    num = num + two * (av(av(wx[0][0], wx[0][1]), av(wx[1][0], wx[1][1])) * ux) * s13;
    num = num + two * (av(av(uz[0][0], uz[1][0]), av(uz[0][1], uz[1][1])) * wz) * s13;
    num = num + two * av(av(uy[0][0], uy[1][0]) * av(wy[0][0], wy[0][1]), av(uy[0][1], uy[1][1]) * av(wy[1][0], wy[1][1])) * s13;
    // S23 (subgrid.f90:835-866)
    num = num + two * (av(av(wy[0][0], wy[0][1]), av(wy[1][0], wy[1][1])) * vy) * s23;
    num = num + two * (av(av(vz[0][0], vz[1][0]), av(vz[0][1], vz[1][1])) * wz) * s23;
    num = num + two * av(av(vx[0][0], vx[0][1]) * av(wx[0][0], wx[0][1]), av(vx[1][0], vx[1][1]) * av(wx[1][0], wx[1][1])) * s23;
    const T v = -T(0.3) * num / den;
    return v > T(0) ? v : T(0);
}

template <typename T> struct AmdMinB { static constexpr int v = sizeof(T) == 4 ? 2 : 1; };

// nu_t at the canonical cells and at every duplicate / ghost position that
// the periodic copies (boundary_conditions.f90:87-244) and the wall rule
// (subgrid.f90:866-876) fill from them; one partial sum of the canonical
// values per (row j, block) for avg_nu_t (subgrid.f90:877-879).
template <typename T>
__global__ void __launch_bounds__(AMD_TX *AMD_TY, AmdMinB<T>::v) k_amd(GeoT<T> g, RcpT<T> rc, Fld<T> U, Fld<T> V,
                                                                      Fld<T> W, Fld<T> nt, int wall_rule,
                                                                      const DevScal *ds, double *part, int kc_len) {
    constexpr int TX = AMD_TX, TY = AMD_TY, SX = TX + 2, SY = TY + 2, NP = SX * SY, NT = TX * TY;
    constexpr int NL = (NP + NT - 1) / NT;
    __shared__ T ring[3][3][NP];  // [plane slot][field U V W][tile]
    const int nx = g.nx, ny = g.ny, nz = g.nz, nxg = g.nxg, nyg = g.nyg, nzg = g.nzg, nxp = g.nxp, nzp = g.nzp;
    const int i0 = 2 + blockIdx.x * TX, j0 = 2 + blockIdx.y * TY;
    const int kb = 2 + blockIdx.z * kc_len, ke = min(kb + kc_len - 1, nzp + 1);
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int i = i0 + tx, j = j0 + ty;
    const bool on = i <= nxp + 1 && j <= nyg - 1;
    const Sp<T> sx{g.x, rc.dx}, sxg{g.xg, rc.dxg}, sy{g.y, rc.dy}, syg{g.yg, rc.dyg}, sz{g.z, rc.dz}, szg{g.zg, rc.dzg};
    // wall rule 2: -nu_t(2) + 2 0.38 dPdx^(1/2) (y(2)-y(1))/2
    T add = T(0);
    if (wall_rule == 2) add = (T)(2.0 * 0.38 * sqrt(ds->dPdx) * ((double)g.y[2] - (double)g.y[1]) / 2.0);
    int eia[NL], eja[NL], erem[NL];
#pragma unroll
    for (int qq = 0; qq < NL; qq++) {
        const int rem = threadIdx.x + qq * NT;
        erem[qq] = rem;
        const int sy_ = rem / SX, sx_ = rem - sy_ * SX;
        eia[qq] = i0 + sx_ - 1;
        eja[qq] = j0 + sy_ - 1;
    }
    T pre[3][NL];
    auto fetch = [&](int k) {
#pragma unroll
        for (int qq = 0; qq < NL; qq++) {
            const int ia = eia[qq], ja = eja[qq];
            const bool in = erem[qq] < NP;
            pre[0][qq] = (in && ia <= nx && ja <= nyg && k <= nzg) ? U(ia, ja, k) : T(0);
            pre[1][qq] = (in && ia <= nxg && ja <= ny && k <= nzg) ? V(ia, ja, k) : T(0);
            pre[2][qq] = (in && ia <= nxg && ja <= nyg && k <= nz) ? W(ia, ja, k) : T(0);
        }
    };
    auto commit = [&](int slot) {
#pragma unroll
        for (int qq = 0; qq < NL; qq++)
            if (erem[qq] < NP) {
#pragma unroll
                for (int f = 0; f < 3; f++) ring[slot][f][erem[qq]] = pre[f][qq];
            }
    };
    fetch(kb - 1);
    commit(0);
    fetch(kb);
    commit(1);
    fetch(kb + 1);
    commit(2);
    __syncthreads();
    // duplicate / ghost images of this column
    const int ix1 = i + nxp <= nxp + 3 ? i + nxp : 0, ix2 = i - nxp >= 1 ? i - nxp : 0;
    const int jg = j == 2 ? 1 : (j == nyg - 1 ? nyg : 0);
    float accf = 0.f;
    double accd = 0.0;
    int sm1 = 0, s0 = 1, sp1 = 2;
    for (int k = kb; k <= ke; k++) {
        if (k + 1 <= ke) fetch(k + 2);  // in flight during this plane's work
        if (on) {
            AmdRing<T> aU, aV, aW;
            aU.b[0] = ring[sm1][0]; aU.b[1] = ring[s0][0]; aU.b[2] = ring[sp1][0];
            aV.b[0] = ring[sm1][1]; aV.b[1] = ring[s0][1]; aV.b[2] = ring[sp1][1];
            aW.b[0] = ring[sm1][2]; aW.b[1] = ring[s0][2]; aW.b[2] = ring[sp1][2];
            aU.i0 = aV.i0 = aW.i0 = i0;
            aU.j0 = aV.j0 = aW.j0 = j0;
            aU.kc = aV.kc = aW.kc = k;
            const T v = amd_point<T, AmdRing<T>>(sx, sxg, sy, syg, sz, szg, aU, aV, aW, i, j, k);
            if constexpr (sizeof(T) == 8) accd += v;
            else accf += v;
            const T gv = wall_rule == 0 ? v : -v + add;
            const int kz1 = k + nzp <= nzp + 3 ? k + nzp : 0, kz2 = k - nzp >= 1 ? k - nzp : 0;
            const int ixs[3] = {i, ix1, ix2}, kzs[3] = {k, kz1, kz2};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (!ixs[a]) continue;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if (!kzs[c]) continue;
                    nt(ixs[a], j, kzs[c]) = v;
                    if (jg) nt(ixs[a], jg, kzs[c]) = gv;
                }
            }
        }
        __syncthreads();               // plane k-1 no longer read
        if (k + 1 <= ke) commit(sm1);  // plane k+2 into the freed slot
        __syncthreads();
        const int t0 = sm1;
        sm1 = s0;
        s0 = sp1;
        sp1 = t0;
    }
    double acc = sizeof(T) == 8 ? accd : (double)accf;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    const int nparts = gridDim.x * gridDim.z;
    if (tx == 0 && j <= nyg - 1) part[(long)(j - 2) * nparts + blockIdx.z * gridDim.x + blockIdx.x] = acc;
}

// avg_nu_t(j) = plane mean of the canonical values, rows 2..nyg-1; rows 1
// and nyg are left as they were (subgrid.f90:877-879).  One warp per row.
__global__ void k_amd_avg(const double *part, int nparts, int nyg, double norm, double *avg) {
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) + 2;
    if (j > nyg - 1) return;
    double a = 0.0;
    for (int qq = lane; qq < nparts; qq += 32) a += part[(long)(j - 2) * nparts + qq];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) {
        const double c = a / norm;
        avg[j] = c;
        ((float *)(avg + nyg + 2))[j] = (float)c;  // FP32 copy
    }
}

}  // namespace

// z chunks of the AMD pass: the count that minimises (waves of resident
// blocks) x (planes per chunk + the 2 halo planes a chunk loads again)
void amd_plan(int esz, int nxp, int nym, int nzp, int sms, int *nkc, int *nparts) {
    int per = 1;
    if (esz == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_amd<float>, AMD_TX * AMD_TY, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_amd<double>, AMD_TX * AMD_TY, 0);
    const long tiles = (long)cdiv(nxp, AMD_TX) * cdiv(nym, AMD_TY), res = (long)(per < 1 ? 1 : per) * sms;
    long best = 1;
    double best_cost = 1e300;
    for (long n = 1; n <= std::max(1L, (long)nzp / 4); n++) {
        const double waves = (double)((tiles * n + res - 1) / res);
        const double cost = waves * ((double)cdiv(nzp, n) + 2.0);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = n;
        }
    }
    const int kc_len = cdiv(nzp, best);
    *nkc = cdiv(nzp, kc_len);
    *nparts = cdiv(nxp, AMD_TX) * *nkc;
}

template <typename T>
int launch_amd(cf_ctx *ctx, int b) {
    ctx->nut_lazy = false;
    GeoT<T> g = geo_of<T>(ctx);
    Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    Fld<T> nt = make_fld<T>(ctx->nut, ctx->nxg, ctx->nyg);
    const int nkc = ctx->amd_nkc, kc_len = cdiv(ctx->nzp, nkc);
    const dim3 grd(cdiv(ctx->nxp, AMD_TX), cdiv(ctx->nym, AMD_TY), nkc);
    k_amd<T><<<grd, AMD_TX * AMD_TY, 0, ctx->st>>>(g, rcp_of<T>(ctx), U, V, W, nt, ctx->prm.Dirichlet_nu_t, ctx->ds,
                                                    ctx->dsm_part, kc_len);
    count_launch(ctx, "k_amd");
    // nothing in the step reads avg_nu_t of the AMD model (the reference
    // marks it "not used"): the plane means are formed from the partials of
    // the last pass when they are asked for
    ctx->amd_nparts = (int)(grd.x * grd.z);
    ctx->amd_avg_pending = true;
    CF_CUDA(cudaGetLastError());
    return 0;
}

int amd_partials_for(cf_ctx *ctx, int nkc) { return cdiv(ctx->nxp, AMD_TX) * cdiv(ctx->nzp, cdiv(ctx->nzp, nkc)); }

int launch_avg_nu_t_flush(cf_ctx *ctx) {
    if (!ctx->amd_avg_pending) return 0;
    k_amd_avg<<<cdiv(ctx->nym, 8), 256, 0, ctx->st>>>(ctx->dsm_part, ctx->amd_nparts, ctx->nyg,
                                                      (double)ctx->nxp * ctx->nzp, ctx->avg_nu_t);
    count_launch(ctx, "k_amd_avg");
    ctx->amd_avg_pending = false;
    CF_CUDA(cudaGetLastError());
    return 0;
}

template int launch_amd<double>(cf_ctx *, int);
template int launch_amd<float>(cf_ctx *, int);
