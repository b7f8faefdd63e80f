// k_dsm.cu -- dynamic Smagorinsky eddy viscosity, subgrid.f90:376-538.
//
// Quantities the reference keeps only as periodic copies are computed at the
// canonical cells (i = 2..nx-1, j = 2..nyg-1, k = 2..nz-1) and read through
// the periodic wrap; U, V, W are always read at their actual indices, because
// with the equilibrium wall model their wall ghost rows are not periodic at
// the duplicate planes.  Plane sums (subgrid.f90:497-513) run over
// i = 2..nxg-1, k = 2..nzg-1 like the reference, i.e. the duplicate column
// i = nxg-1 and row k = nzg-1 (copies of i = 2, k = 2) are counted twice;
// here that is a weight 2 on the canonical column/row 2.
#include <cuda.h>  // CUtensorMap (the encoder is reached through the runtime's driver entry point)

#include <algorithm>
#include <cstring>
#include <mutex>

#include "cf_internal.cuh"

enum { Q_UC = 0, Q_VC, Q_WC, Q_UU, Q_VV, Q_WW, Q_UV, Q_UW, Q_VW, Q_SS1, Q_SS2, Q_SS3, Q_SS4, Q_SS5, Q_SS6, Q_S, NQ };

struct Can {
    int nxp, nym, nzp;
    long n;
    __device__ __forceinline__ long operator()(int i, int j, int k) const {
        return (long)(i - 2) + (long)nxp * ((j - 2) + (long)nym * (k - 2));
    }
};

// Stage A: centre velocities, products and |S| S_ij at canonical centres.
template <typename T>
__global__ void k_dsm_a(GeoT<T> g, RcpT<T> rc, Fld<T> U, Fld<T> V, Fld<T> W, T *q, Can c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
    int k = blockIdx.z + 2;
    if (i > g.nx - 1 || j > g.nyg - 1) return;
    long o = c(i, j, k), n = c.n;
    const T h = T(0.5);
    // subgrid.f90:392-394
    T uc = h * (U(i - 1, j, k) + U(i, j, k));
    T vc = h * (V(i, j - 1, k) + V(i, j, k));
    T wc = h * (W(i, j, k - 1) + W(i, j, k));
    q[o + Q_UC * n] = uc;
    q[o + Q_VC * n] = vc;
    q[o + Q_WC * n] = wc;
    q[o + Q_UU * n] = uc * uc;
    q[o + Q_VV * n] = vc * vc;
    q[o + Q_WW * n] = wc * wc;
    q[o + Q_UV * n] = uc * vc;
    q[o + Q_UW * n] = uc * wc;
    q[o + Q_VW * n] = vc * wc;
    T s[6], S;
    sij_point<T>(g, rc, U, V, W, i, j, k, s, S);
#pragma unroll
    for (int a = 0; a < 6; a++) q[o + (Q_SS1 + a) * n] = S * s[a];
    q[o + Q_S * n] = S;
}

// Stages B and D: L_ij = hat(ui uj) - hat(ui) hat(uj) and hat(|S| S_ij)
// (the filter of 15 canonical quantities), then M_ij = 4 |S(Uf)| S_ij(Uf) -
// hat(|S| S_ij) and the plane partial sums of L.M and M.M
// (subgrid.f90:429-513).  A block owns a DB_X x DB_Y tile of (i, j) and
// marches along z over a chunk of planes: each plane of the 15 quantities
// (tile plus one halo cell, periodic in x, rows clamped to the interior) is
// gathered into a shared-memory buffer while an earlier one is filtered; the
// FP32 kernel filters it in y by a column pass and in x at its point (the
// FP64 kernel with a 9-point stencil at its point) and spreads the result
// over the z accumulators of planes r-1, r, r+1 (weights 1/6, 2/3, 1/6), so
// that plane r-1 is complete once plane r is in.  The filtered velocities
// Uf, Vf, Wf (stage C) are read at their actual indices, while the next
// plane's copies are in flight.  The plane sums (float-float in the FP32
// kernel) count the duplicate column and plane as weight 2 on i = 2 and
// k = 2 (the reference's loops run over i = 2..nxg-1, k = 2..nzg-1).
//
// Two gathers: per-element cp.async copies into two buffers (any nxp, FP64
// and FP32), and for FP32 with nxp a multiple of 4 one tensor copy (TMA) per
// plane into three buffers, two planes in flight.  The tensor copy is a 4D
// box of x 40, y 10, z 1 and all 15 quantities; its x origin is 4 columns
// before the tile's halo column (16-byte aligned), its y origin the row
// before the tile.  Rows outside 0..nym-1 arrive as zeros and meet only the
// zero weights of the one-sided y filter (the cp.async gather clamps them
// instead: the products are 0 either way); the periodic halo columns
// (canonical -1 -> nxp-1 at the first tile, nxp -> 0 at the last) arrive as
// zeros too and are overwritten from registers loaded before the wait.
constexpr int DB_X = 32, DB_Y = 8, DB_NQ = 15;
constexpr int DBT_BX = DB_X + 8, DBT_BY = DB_Y + 2, DBT_OX = 3;  // box extents; column of halo column 0
constexpr int DBT_PLANE = DBT_BX * DBT_BY;                        // floats per quantity in a buffer
constexpr unsigned DBT_BYTES = DB_NQ * DBT_PLANE * 4;             // 24000 bytes per plane
constexpr int DBT_STRIDE = (int)((DBT_BYTES + 127) / 128 * 128);  // buffer stride: 128-byte aligned
constexpr int DBT_NB = 3;                                         // buffers: the plane filtered + 2 in flight
constexpr int DBT_NFIX = 2 * DB_NQ * DBT_BY;                      // periodic halo values of a plane
// a plane copy is given up after this long (it completes within microseconds)
constexpr uint64_t DBT_WAIT_NS = 200000000ull;

// asynchronous global -> shared copies of single elements (the plane gather
// of the next z plane runs while the current one is filtered)
template <int B>
__device__ __forceinline__ void cp_async_elem(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
__device__ __forceinline__ uint32_t sh_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t dbt_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}
// wait for phase `parity` of the mbarrier at shared address `mb`; false when
// DBT_WAIT_NS passed first
__device__ __forceinline__ bool dbt_wait(uint32_t mb, uint32_t parity) {
    const uint64_t t0 = dbt_ns();
    for (long it = 0; it < (1L << 24); it++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(mb), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & 31) == 31 && dbt_ns() - t0 > DBT_WAIT_NS) return false;
    }
    return false;
}
// dynamic shared memory of k_dsm_b: the plane buffers of the 15 quantities
template <typename T, bool TMA>
constexpr size_t dsm_b_smem() {
    return TMA ? (size_t)DBT_NB * DBT_STRIDE + 128 : (size_t)2 * DB_NQ * (DB_X + 2) * (DB_Y + 2) * sizeof(T);
}

// TMA: the tensor-copy gather (FP32, nxp a multiple of 4; tm maps the 15
// quantities of q as x nxp, y nym, z nzp, quantity 15).  skip_first (a test
// hook): plane kb-1 is not copied, so its wait expires and the block stops.
// A wait that expired is counted in ds->n_wait; the block's copies still in
// flight are waited for (with the same limit) before it returns.
template <typename T, bool TMA>
__global__ void __launch_bounds__(DB_X *DB_Y) k_dsm_b(const __grid_constant__ CUtensorMap tm, const T *__restrict__ q,
                                                      GeoT<T> g, RcpT<T> rc, Fld<T> Uf, Fld<T> Vf, Fld<T> Wf, Can c,
                                                      int nyg, int kc_len, double *part, int nchunk, DevScal *ds,
                                                      int skip_first) {
    static_assert(!TMA || sizeof(T) == 4, "the tensor-copy gather is the FP32 kernel's");
    constexpr int SX = DB_X + 2, SY = DB_Y + 2, NP = SX * SY;
    // a buffer: DB_NQ quantities of PQ elements, rows of pitch PX, halo
    // column 0 at column OX
    constexpr int PX = TMA ? DBT_BX : SX, PQ = TMA ? DBT_PLANE : NP, OX = TMA ? DBT_OX : 0;
    constexpr int NB = TMA ? DBT_NB : 2, BS = TMA ? DBT_STRIDE / (int)sizeof(T) : DB_NQ * NP;
    extern __shared__ __align__(16) unsigned char dsmb_raw[];
    // tensor-copy destinations are 128-byte aligned
    T *plb = (T *)(dsmb_raw + (TMA ? (128 - (sh_u32(dsmb_raw) & 127)) & 127 : 0));  // [NB][DB_NQ][PQ]
    __shared__ __align__(8) uint64_t bar[NB];
    // the plane filtered in y, rows of the tile (FP32: within 48 KB of static
    // shared memory with the plane; the FP64 kernel filters from the plane)
    constexpr bool COLS = sizeof(T) == 4;
    __shared__ T cl[COLS ? DB_NQ : 1][DB_Y][SX];
    __shared__ double red[2][DB_X * DB_Y];
    const int tx = threadIdx.x % DB_X, ty = threadIdx.x / DB_X;
    const int i0 = 2 + blockIdx.x * DB_X, j0 = 2 + blockIdx.y * DB_Y;
    const int kb = 2 + blockIdx.z * kc_len, ke = min(kb + kc_len - 1, c.nzp + 1);
    const int i = i0 + tx, j = j0 + ty;
    const bool own = i <= c.nxp + 1 && j <= nyg - 1;
    const long n = c.n;
    const T f6 = T(1.0 / 6.0), f23 = T(2.0 / 3.0), f13 = T(1.0 / 3.0);
    const T fw[3] = {f6, f23, f6};
    T accp[DB_NQ], accc[DB_NQ];  // planes r-1 (two contributions in) and r (one)
#pragma unroll
    for (int qq = 0; qq < DB_NQ; qq++) accp[qq] = accc[qq] = T(0);
    // plane sums of this thread: FP64 in the FP64 path, float-float in the
    // split path (an FP64 instruction per cell costs dozens of FP32 ones here)
    double sl = 0.0, smm = 0.0;
    float slh = 0.f, sll = 0.f, smh = 0.f, sml = 0.f;
    // gather of plane r into buffer b: one tensor copy issued by thread 0
    // (TMA), or one group of per-element asynchronous copies (tile plus one
    // halo cell, periodic in x, rows clamped to the interior)
    auto issue = [&](int r, int b) {
        const int rc_ = wrapn(r, c.nzp);
        if constexpr (TMA) {
            if (threadIdx.x == 0) {
                const uint32_t mb = sh_u32(&bar[b]);
                const int x0 = blockIdx.x * DB_X - 4, y0 = blockIdx.y * DB_Y - 1, z0 = rc_ - 2;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(DBT_BYTES)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
                    "[%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(sh_u32(plb + b * BS)),
                    "l"(reinterpret_cast<uint64_t>(&tm)), "r"(x0), "r"(y0), "r"(z0), "r"(0), "r"(mb)
                    : "memory");
            }
        } else {
            for (int e = threadIdx.x; e < NP; e += DB_X * DB_Y) {
                const int sy = e / SX, sx = e - sy * SX;
                // columns past the domain's last halo are never read: clamp them in range
                const int ii = wrapn(min(i0 + sx - 1, c.nxp + 2), c.nxp), jj = min(max(j0 + sy - 1, 2), nyg - 1);
                const long o = c(ii, jj, rc_);
#pragma unroll
                for (int qq = 0; qq < DB_NQ; qq++) cp_async_elem<sizeof(T)>(plb + (b * DB_NQ + qq) * NP + e, q + o + qq * n);
            }
            cp_async_commit();
        }
    };
    // periodic halo columns of the tensor-copy gather: column 0 of the first
    // tile holds canonical nxp-1, column sxr = nxp - 32 bx + 1 (when inside
    // the tile's 34 columns) canonical 0.  Task t < DBT_NFIX: side t / 150,
    // quantity (t % 150) / 10, row t % 10; rows outside 0..nym-1 stay 0.
    const int sxr = c.nxp - (int)blockIdx.x * DB_X + 1;
    const bool fixl = TMA && blockIdx.x == 0, fixr = TMA && sxr >= 1 && sxr <= SX - 1;
    const bool fixb = fixl || fixr;  // block-uniform
    constexpr int NFT = (DBT_NFIX + DB_X * DB_Y - 1) / (DB_X * DB_Y);
    if constexpr (TMA) {
        if (threadIdx.x == 0) {
#pragma unroll
            for (int b = 0; b < NB; b++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(sh_u32(&bar[b])));
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        }
        __syncthreads();
        for (int p = 0; p < NB - 1 && kb - 1 + p <= ke + 1; p++)
            if (!(skip_first && p == 0)) issue(kb - 1 + p, p);
    } else {
        issue(kb - 1, 0);
    }
    int rfail = 0;
    for (int r = kb - 1; r <= ke + 1; r++) {
        const int u = r - (kb - 1), cur = u % NB;
        T(*pl)[PQ] = (T(*)[PQ])(plb + cur * BS);
        __syncthreads();  // plane r-1 (the buffer refilled next) is no longer read
        if constexpr (TMA) {
            if (r + NB - 1 <= ke + 1) issue(r + NB - 1, (u + NB - 1) % NB);
        } else {
            if (r + 1 <= ke + 1) issue(r + 1, cur ^ 1);
        }
        // the periodic halo values of plane r, loaded before the wait
        float fxv[NFT];
        int fxo[NFT];
        if constexpr (TMA) {
            if (fixb) {
                const int z = wrapn(r, c.nzp) - 2;
#pragma unroll
                for (int f = 0; f < NFT; f++) {
                    const int t = threadIdx.x + f * DB_X * DB_Y, side = t / (DB_NQ * DBT_BY);
                    const int qq = (t % (DB_NQ * DBT_BY)) / DBT_BY, sy = t % DBT_BY, y = (int)blockIdx.y * DB_Y - 1 + sy;
                    const bool on = t < DBT_NFIX && (side == 0 ? fixl : fixr) && y >= 0 && y < c.nym;
                    fxo[f] = on ? qq * PQ + sy * PX + OX + (side == 0 ? 0 : sxr) : -1;
                    fxv[f] = on ? (float)q[(long)qq * n + (side == 0 ? c.nxp - 1 : 0) + (long)c.nxp * (y + (long)c.nym * z)]
                                : 0.f;
                }
            }
        }
        // S_ij of the filtered velocities at the output plane k = r-1
        // (fil_size**2 = 4 in M, subgrid.f90:156, 463), read from global
        // memory while the plane copies are in flight
        const int k = r - 1;
        const bool outp = own && k >= kb;
        T sf[6], Sf = T(0);
        if (outp) sij_point<T>(g, rc, Uf, Vf, Wf, i, j, k, sf, Sf);
        if constexpr (TMA) {
            // plane r has landed (every thread observes the phase; the block
            // agrees on the outcome)
            const bool ok = dbt_wait(sh_u32(&bar[cur]), (u / NB) & 1);
            if (!__syncthreads_and(ok)) {
                rfail = r;
                break;
            }
            if (fixb) {
#pragma unroll
                for (int f = 0; f < NFT; f++)
                    if (fxo[f] >= 0) ((float *)pl[0])[fxo[f]] = fxv[f];
                // these generic writes precede the tensor copy that refills the buffer
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                __syncthreads();
            }
        } else {
            if (r + 1 <= ke + 1) cp_async_wait<1>();  // this thread's copies of plane r are done
            else cp_async_wait<0>();
            __syncthreads();  // and every thread's
        }
        // y filter, one (quantity, column) per task: the column's SY values
        // give the DB_Y filtered rows (one-sided at rows 2 and nyg-1)
        if constexpr (COLS) {
        for (int t = threadIdx.x; t < DB_NQ * SX; t += DB_X * DB_Y) {
            const int qq = t / SX, sx = t - qq * SX;
            T col[SY];
#pragma unroll
            for (int sy = 0; sy < SY; sy++) col[sy] = pl[qq][sy * PX + sx + OX];
#pragma unroll
            for (int oy = 0; oy < DB_Y; oy++) {
                const int jr = j0 + oy;
                const T rm = jr == 2 ? T(0) : (jr == nyg - 1 ? f13 : f6), rp = jr == 2 ? f13 : (jr == nyg - 1 ? T(0) : f6);
                cl[qq][oy][sx] = rm * col[oy] + f23 * col[oy + 1] + rp * col[oy + 2];
            }
        }
        __syncthreads();
        }
        if (!own) continue;
        // y weights of this row for the FP64 kernel (one-sided at rows 2 and nyg-1)
        const T wm = j == 2 ? T(0) : (j == nyg - 1 ? f13 : f6), wp = j == 2 ? f13 : (j == nyg - 1 ? T(0) : f6);
        const int e = (ty + 1) * PX + tx + 1 + OX;
        T fq[DB_NQ];
#pragma unroll
        for (int qq = 0; qq < DB_NQ; qq++) {
            T a = T(0);
#pragma unroll
            for (int d = -1; d <= 1; d++) {
                if constexpr (COLS) a += fw[d + 1] * cl[qq][ty][tx + 1 + d];
                else a += fw[d + 1] * (wm * pl[qq][e + d - PX] + f23 * pl[qq][e + d] + wp * pl[qq][e + d + PX]);
            }
            fq[qq] = accp[qq] + f6 * a;  // plane r-1, complete
            accp[qq] = accc[qq] + f23 * a;
            accc[qq] = f6 * a;
        }
        if (!outp) continue;
        const T fu = fq[0], fv = fq[1], fwv = fq[2];
        const T pa[6] = {fu, fv, fwv, fu, fu, fv}, pb[6] = {fu, fv, fwv, fv, fwv, fwv};
        T L[6], M[6];
#pragma unroll
        for (int a = 0; a < 6; a++) {
            L[a] = fq[3 + a] - pa[a] * pb[a];
            M[a] = T(4) * Sf * sf[a] - fq[9 + a];
        }
        const T lm = (L[0] * M[0] + L[1] * M[1] + L[2] * M[2] + T(2) * (L[3] * M[3] + L[4] * M[4] + L[5] * M[5]));
        const T mm = (M[0] * M[0] + M[1] * M[1] + M[2] * M[2] + T(2) * (M[3] * M[3] + M[4] * M[4] + M[5] * M[5]));
        if constexpr (sizeof(T) == 4) {
            const float wgt = (i == 2 ? 2.f : 1.f) * (k == 2 ? 2.f : 1.f);  // exact: lm, mm times 1, 2 or 4
            ff_add(slh, sll, wgt * lm);
            ff_add(smh, sml, wgt * mm);
        } else {
            const double wgt = (i == 2 ? 2.0 : 1.0) * (k == 2 ? 2.0 : 1.0);
            sl += wgt * (double)lm;
            smm += wgt * (double)mm;
        }
    }
    if constexpr (TMA) {
        if (rfail) {
            // a plane copy did not arrive in time: count it, wait for the
            // copies still in flight (planes rfail .. rfail + NB - 1) and stop
            if (threadIdx.x == 0) {
                atomicAdd(&ds->n_wait, 1);
                for (int p = rfail; p <= min(rfail + NB - 1, ke + 1); p++) {
                    const int u = p - (kb - 1);
                    if (!(skip_first && u == 0)) dbt_wait(sh_u32(&bar[u % NB]), (u / NB) & 1);
                }
            }
            return;
        }
    }
    if constexpr (sizeof(T) == 4) {
        // one warp per row (DB_X = 32): float-float shuffle tree, lane 0
        // writes (L.M hi, lo, M.M hi, lo)
        if (!own) slh = sll = smh = sml = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float a1 = __shfl_down_sync(0xffffffffu, slh, o), a2 = __shfl_down_sync(0xffffffffu, sll, o);
            const float b1 = __shfl_down_sync(0xffffffffu, smh, o), b2 = __shfl_down_sync(0xffffffffu, sml, o);
            ff_add2(slh, sll, a1, a2);
            ff_add2(smh, sml, b1, b2);
        }
        if (tx == 0 && j <= nyg - 1) {
            const long chunk = (long)blockIdx.z * gridDim.x + blockIdx.x;
            ((float4 *)part)[(long)(j - 2) * nchunk + chunk] = make_float4(slh, sll, smh, sml);
        }
        return;
    }
    // plane partials of this block for row j: the sum over the tile's DB_X threads of the row
    red[0][threadIdx.x] = sl;
    red[1][threadIdx.x] = smm;
    __syncthreads();
    if (tx == 0 && j <= nyg - 1) {
        double a = 0.0, b = 0.0;
        for (int t = 0; t < DB_X; t++) {
            a += red[0][ty * DB_X + t];
            b += red[1][ty * DB_X + t];
        }
        const long chunk = (long)blockIdx.z * gridDim.x + blockIdx.x;
        part[((long)(j - 2) * nchunk + chunk) * 2] = a;
        part[((long)(j - 2) * nchunk + chunk) * 2 + 1] = b;
    }
}

// Stage C: filtered velocities Uf, Vf, Wf (subgrid.f90:431-445) at every
// element of their arrays; ghost and duplicate elements take the value of the
// canonical element (the periodic fills of subgrid.f90:448-458); y one-sided
// at rows 1 and n2.  A z-marching tile kernel: a block owns a 32 x 8 tile of
// (canonical i, j), one raw plane (tile plus one halo cell) in shared memory,
// the next plane's loads in flight in registers while the current one is
// filtered in x and y, the z filter over a register ring of three filtered
// planes; each canonical value is stored to every element that wraps to it.
// (The x-y filter is taken before the z filter, the reverse of the order of
// a 27-point loop over x outermost: the results agree to rounding.)
template <typename T>
__global__ void __launch_bounds__(256) k_dsm_c_t(Fld<T> A, Fld<T> Af, int n1, int n2, int n3, int nxp, int nzp,
                                                 int kc_len) {
    constexpr int TX = 32, TY = 8, SX = TX + 2, SY = TY + 2, NP = SX * SY, NT = TX * TY, NL = (NP + NT - 1) / NT;
    __shared__ T pl[NP];
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int is0 = 2 + blockIdx.x * TX, j0 = 1 + blockIdx.y * TY;
    const int kb = 2 + blockIdx.z * kc_len, ke = min(kb + kc_len - 1, nzp + 1);
    const int is = is0 + tx, j = j0 + ty;
    const bool own = is <= nxp + 1 && j <= n2;
    const T f6 = T(1.0 / 6.0), f23 = T(2.0 / 3.0), f13 = T(1.0 / 3.0);
    T wm, w0, wp;
    if (j == 1) { wm = T(0); w0 = f23; wp = f13; }
    else if (j == n2) { wm = f13; w0 = f23; wp = T(0); }
    else { wm = f6; w0 = f23; wp = f6; }
    // rows 0 and n2+1 of the tile read row 1 and n2 (their weight is 0);
    // columns past the array are never read by an owned point: clamped
    int eidx[NL];
#pragma unroll
    for (int q = 0; q < NL; q++) {
        const int e = threadIdx.x + q * NT, sy = e / SX, sx = e - sy * SX;
        const int ii = min(is0 - 1 + sx, n1), jj = min(max(j0 - 1 + sy, 1), n2);
        eidx[q] = e < NP ? A.idx(ii, jj, 1) : -1;
    }
    T pre[NL];
    auto fetch = [&](int k) {
#pragma unroll
        for (int q = 0; q < NL; q++) pre[q] = eidx[q] >= 0 ? A.p[eidx[q] + (long)A.sz * (k - 1)] : T(0);
    };
    T g2 = T(0), g1 = T(0);  // x-y filtered planes p-2, p-1 at the own point
    fetch(kb - 1);
    for (int p = kb - 1; p <= ke + 1; p++) {
        __syncthreads();  // the previous plane is no longer read
#pragma unroll
        for (int q = 0; q < NL; q++)
            if (eidx[q] >= 0) pl[threadIdx.x + q * NT] = pre[q];
        __syncthreads();
        if (p + 1 <= ke + 1) fetch(p + 1);
        if (!own) continue;
        const int e = (ty + 1) * SX + tx + 1;
        T g = T(0);
#pragma unroll
        for (int a = -1; a <= 1; a++) {
            const T fa = a == 0 ? f23 : f6;
            g += fa * (wm * pl[e + a - SX] + w0 * pl[e + a] + wp * pl[e + a + SX]);
        }
        if (p >= kb + 1) {
            const int ks = p - 1;
            const T v = f6 * g2 + f23 * g1 + f6 * g;
            // every element (i, j, k) with wrapc(i) = is, wrapc(k) = ks
#pragma unroll
            for (int di = -1; di <= 1; di++) {
                const int i = is + di * nxp;
                if (i < 1 || i > n1) continue;
#pragma unroll
                for (int dk = -1; dk <= 1; dk++) {
                    const int k = ks + dk * nzp;
                    if (k < 1 || k > n3) continue;
                    Af(i, j, k) = v;
                }
            }
        }
        g2 = g1;
        g1 = g;
    }
}

// Stage E: avg_nu_t(j) = <LM>/<MM> (subgrid.f90:516-518) and its ghosts.
// <LM>/<MM> per row from the block partial sums: one warp per row, lanes
// over chunks in a fixed order, then the ghost rows (subgrid.f90:515-519).
// nbase: the slots of a row outside the wall-model seam band (the seam
// kernel's slots follow them only in the band's rows; nbase = nchunk when
// there are none)
__global__ void k_dsm_e(const double *part, int nchunk, int nyg, double *avg, int dirichlet, int nbase) {
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) + 2;
    if (j > nyg - 1) return;
    const int nread = seam_row(j, nyg) ? nchunk : nbase;
    double a = 0.0, b = 0.0;
    for (int q = lane; q < nread; q += 32) {
        a += part[((long)(j - 2) * nchunk + q) * 2];
        b += part[((long)(j - 2) * nchunk + q) * 2 + 1];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        float *af = (float *)(avg + nyg + 2);  // FP32 copy for the split path
        const double c = a / b;
        avg[j] = c;
        af[j] = (float)c;
        if (j == 2) {
            avg[1] = dirichlet ? -c : c;
            af[1] = (float)avg[1];
        }
        if (j == nyg - 1) {
            avg[nyg] = dirichlet ? -c : c;
            af[nyg] = (float)avg[nyg];
        }
    }
}
// The same from float-float partials (L.M hi, lo, M.M hi, lo) of the one-pass
// FP32 kernel: the sums in float-float, FP64 only for lane 0's quotient.
__global__ void k_dsm_e_ff(const float4 *part, int nchunk, int nyg, double *avg, int dirichlet, int nbase) {
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) + 2;
    if (j > nyg - 1) return;
    const int nread = seam_row(j, nyg) ? nchunk : nbase;
    float ah = 0.f, al = 0.f, bh = 0.f, bl = 0.f;
    for (int q = lane; q < nread; q += 32) {
        const float4 v = part[(long)(j - 2) * nchunk + q];
        ff_add2(ah, al, v.x, v.y);
        ff_add2(bh, bl, v.z, v.w);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float a1 = __shfl_down_sync(0xffffffffu, ah, o), a2 = __shfl_down_sync(0xffffffffu, al, o);
        const float b1 = __shfl_down_sync(0xffffffffu, bh, o), b2 = __shfl_down_sync(0xffffffffu, bl, o);
        ff_add2(ah, al, a1, a2);
        ff_add2(bh, bl, b1, b2);
    }
    if (lane == 0) {
        float *af = (float *)(avg + nyg + 2);  // FP32 copy for the split path
        const double c = ((double)ah + (double)al) / ((double)bh + (double)bl);
        avg[j] = c;
        af[j] = (float)c;
        if (j == 2) {
            avg[1] = dirichlet ? -c : c;
            af[1] = (float)avg[1];
        }
        if (j == nyg - 1) {
            avg[nyg] = dirichlet ? -c : c;
            af[nyg] = (float)avg[nyg];
        }
    }
}

// Stage F: nu_t = max(-0.5 C(j) |S|, 0) everywhere, periodic copies and the
// wall ghost rule (subgrid.f90:521-536).
template <typename T>
// walls: rows 1, 2, nyg-1, nyg only (blockDim.y = 4, one block row)
__global__ void k_dsm_f(Fld<T> nt, const T *Sq, const double *avg, Can c, int nxg, int nyg, int nzg, int dirichlet,
                        int walls) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (walls) j = threadIdx.y < 2 ? 1 + threadIdx.y : nyg - 3 + threadIdx.y;
    int k = blockIdx.z + 1;
    if (i > nxg || j > nyg) return;
    int jj = j == 1 ? 2 : (j == nyg ? nyg - 1 : j);
    int is = wrapc(i, c.nxp), ks = wrapc(k, c.nzp);
    T a;
    if constexpr (sizeof(T) == 4) a = ((const float *)(avg + nyg + 2))[jj];
    else a = avg[jj];
    T v = T(-0.5) * a * Sq[c(is, jj, ks)];
    v = v > T(0) ? v : T(0);
    if (jj != j && dirichlet) v = -v;
    nt(i, j, k) = v;
}

template <typename T>
__global__ void k_fill(T *p, long n, T v) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = v;
}

// Fills nut from |S| and the plane coefficient when it is held lazily.
template <typename T>
int launch_nut_materialize(cf_ctx *ctx) {
    if (!ctx->nut_lazy) return 0;
    Can c;
    c.nxp = ctx->nxp; c.nym = ctx->nym; c.nzp = ctx->nzp; c.n = (long)ctx->nCan;
    Fld<T> nt = make_fld<T>(ctx->nut, ctx->nxg, ctx->nyg);
    T *q = (T *)ctx->dsm_q;
    k_dsm_f<T><<<dim3(cdiv(ctx->nxg, 32), cdiv(ctx->nyg, 4), ctx->nzg), dim3(32, 4, 1), 0, ctx->st>>>(
        nt, q + Q_S * c.n, ctx->avg_nu_t, c, ctx->nxg, ctx->nyg, ctx->nzg, ctx->prm.Dirichlet_nu_t == 1, 0);
    count_launch(ctx, "k_dsm_f");
    ctx->nut_lazy = false;
    CF_CUDA(cudaGetLastError());
    return 0;
}

// nu_t of the wall rows and their neighbours (j = 1, 2, nyg-1, nyg), the
// only rows the wall model reads; the rest of the field stays lazy (its
// other readers materialise it).
template <typename T>
int launch_nut_wall_rows(cf_ctx *ctx) {
    if (!ctx->nut_lazy) return 0;
    Can c;
    c.nxp = ctx->nxp; c.nym = ctx->nym; c.nzp = ctx->nzp; c.n = (long)ctx->nCan;
    Fld<T> nt = make_fld<T>(ctx->nut, ctx->nxg, ctx->nyg);
    k_dsm_f<T><<<dim3(cdiv(ctx->nxg, 32), 1, ctx->nzg), dim3(32, 4, 1), 0, ctx->st>>>(
        nt, (T *)ctx->dsm_q + Q_S * c.n, ctx->avg_nu_t, c, ctx->nxg, ctx->nyg, ctx->nzg,
        ctx->prm.Dirichlet_nu_t == 1, 1);
    count_launch(ctx, "k_dsm_f");
    CF_CUDA(cudaGetLastError());
    return 0;
}

template <typename T>
int launch_nut_zero(cf_ctx *ctx) {
    ctx->nut_lazy = false;
    k_fill<T><<<cdiv(ctx->nC, 256), 256, 0, ctx->st>>>((T *)ctx->nut, (long)ctx->nC, T(0));
    count_launch(ctx, "k_fill");
    k_fill<double><<<1, 256, 0, ctx->st>>>(ctx->avg_nu_t, ctx->nyg + 1, 0.0);
    count_launch(ctx, "k_fill");
    CF_CUDA(cudaGetLastError());
    return 0;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult qr = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) ==
                cudaSuccess &&
            qr == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

// Whether the multi-pass filter kernel gathers its planes with tensor copies:
// FP32, nxp a multiple of 4 (16-byte strides and x origins), at least 40 x 10
// canonical cells per plane (the box), not switched off (dsm_unfused 2).  The
// tensor map of the 15 quantities of dsm_q is encoded on the first call.
bool dsmb_tma(cf_ctx *ctx) {
    if (ctx->dsmb_map_state == 0) {
        ctx->dsmb_map_state = -1;
        EncodeTiledFn fn = encode_tiled();
        if (ctx->esz == 4 && ctx->nxp % 4 == 0 && ctx->nxp >= DBT_BX && ctx->nym >= DBT_BY && fn) {
            CUtensorMap m;
            const cuuint64_t dims[4] = {(cuuint64_t)ctx->nxp, (cuuint64_t)ctx->nym, (cuuint64_t)ctx->nzp, DB_NQ};
            const cuuint64_t strides[3] = {(cuuint64_t)ctx->nxp * 4, (cuuint64_t)ctx->nxp * ctx->nym * 4,
                                           (cuuint64_t)ctx->nCan * 4};
            const cuuint32_t box[4] = {DBT_BX, DBT_BY, 1, DB_NQ}, es[4] = {1, 1, 1, 1};
            if (fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, ctx->dsm_q, dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS) {
                static_assert(sizeof(m) == sizeof(ctx->dsmb_map), "tensor map storage");
                std::memcpy(ctx->dsmb_map, &m, sizeof(m));
                ctx->dsmb_map_state = 1;
            }
        }
    }
    return ctx->dsmb_map_state == 1 && ctx->prm.dsm_unfused != 2;
}

template <typename T>
int launch_dsm(cf_ctx *ctx, int b) {
    int dir = ctx->prm.Dirichlet_nu_t == 1;
    Can c;
    c.nxp = ctx->nxp; c.nym = ctx->nym; c.nzp = ctx->nzp; c.n = (long)ctx->nCan;
    dim3 blk(32, 4, 1);
    if (ctx->use_fused_dsm && ctx->state_periodic && (ctx->prm.iwall_model == 0 || ctx->prm.iwall_model == 3)) {
        // one pass: |S| and the plane partial sums (k_dsm_fused.cu); with the
        // wall model the seam band is computed by k_dsm_seam
        int rc = ctx->prm.iwall_model == 0 ? launch_dsm_fused<T>(ctx, b) : launch_dsm_fused_wm<T>(ctx, b);
        if (rc) return rc;
        const int nch = ctx->dsm_nchunk_fused, nb = ctx->dsm_nchunk_base;
        if (sizeof(T) == 4)  // float-float partials of the FP32 kernel
            k_dsm_e_ff<<<cdiv(ctx->nym, 8), 256, 0, ctx->st>>>((const float4 *)ctx->dsm_part, nch, ctx->nyg,
                                                                ctx->avg_nu_t, dir, nb);
        else
            k_dsm_e<<<cdiv(ctx->nym, 8), 256, 0, ctx->st>>>(ctx->dsm_part, nch, ctx->nyg, ctx->avg_nu_t, dir, nb);
        count_launch(ctx, "k_dsm_e");
        ctx->nut_lazy = true;  // nu_t = max(-C(j)|S|/2, 0) is formed by its readers
        CF_CUDA(cudaGetLastError());
        return 0;
    }
    ctx->nut_lazy = false;
    GeoT<T> g = geo_of<T>(ctx);
    Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    T *q = (T *)ctx->dsm_q;
    const RcpT<T> rc = rcp_of<T>(ctx);
    dim3 grdc(cdiv(ctx->nxp, 32), cdiv(ctx->nym, 4), ctx->nzp);
    k_dsm_a<T><<<grdc, blk, 0, ctx->st>>>(g, rc, U, V, W, q, c);
    count_launch(ctx, "k_dsm_a");
    Fld<T> Uf = make_fld<T>(ctx->Uf, ctx->nx, ctx->nyg);
    Fld<T> Vf = make_fld<T>(ctx->Vf, ctx->nxg, ctx->ny);
    Fld<T> Wf = make_fld<T>(ctx->Wf, ctx->nxg, ctx->nyg);
    {
        // z chunks of 16 canonical planes
        const int kc = 16, nkc = cdiv(ctx->nzp, kc), ntx = cdiv(ctx->nxp, 32);
        k_dsm_c_t<T><<<dim3(ntx, cdiv(ctx->nyg, 8), nkc), 256, 0, ctx->st>>>(U, Uf, ctx->nx, ctx->nyg, ctx->nzg, ctx->nxp, ctx->nzp, kc);
        k_dsm_c_t<T><<<dim3(ntx, cdiv(ctx->ny, 8), nkc), 256, 0, ctx->st>>>(V, Vf, ctx->nxg, ctx->ny, ctx->nzg, ctx->nxp, ctx->nzp, kc);
        k_dsm_c_t<T><<<dim3(ntx, cdiv(ctx->nyg, 8), nkc), 256, 0, ctx->st>>>(W, Wf, ctx->nxg, ctx->nyg, ctx->nz, ctx->nxp, ctx->nzp, kc);
    }
    count_launch(ctx, "k_dsm_c_t"); count_launch(ctx, "k_dsm_c_t"); count_launch(ctx, "k_dsm_c_t");
    int nchunk;
    {
        // z chunks planned at context creation (dsm_b_plan), within the plane-partial slots
        const int ntx = cdiv(ctx->nxp, DB_X);
        long nkc = std::max(1L, std::min((long)std::max(ctx->dsmb_nkc, 1), (long)ctx->dsm_part_nch / ntx));
        const int kc_len = cdiv(ctx->nzp, nkc);
        const int nz_chunks = cdiv(ctx->nzp, kc_len);
        nchunk = ntx * nz_chunks;
        const dim3 grd(ntx, cdiv(ctx->nym, DB_Y), nz_chunks);
        CUtensorMap tm;
        if (dsmb_tma(ctx)) {
            std::memcpy(&tm, ctx->dsmb_map, sizeof(tm));
            k_dsm_b<float, true><<<grd, DB_X * DB_Y, dsm_b_smem<float, true>(), ctx->st>>>(
                tm, (const float *)q, geo_of<float>(ctx), rcp_of<float>(ctx), make_fld<float>(ctx->Uf, ctx->nx, ctx->nyg),
                make_fld<float>(ctx->Vf, ctx->nxg, ctx->ny), make_fld<float>(ctx->Wf, ctx->nxg, ctx->nyg), c, ctx->nyg,
                kc_len, ctx->dsm_part, nchunk, ctx->ds, ctx->dsmb_skip_first);
        } else {
            std::memset(&tm, 0, sizeof(tm));  // not read by the per-element gather
            k_dsm_b<T, false><<<grd, DB_X * DB_Y, dsm_b_smem<T, false>(), ctx->st>>>(
                tm, q, g, rc, Uf, Vf, Wf, c, ctx->nyg, kc_len, ctx->dsm_part, nchunk, ctx->ds, 0);
        }
        count_launch(ctx, "k_dsm_b");
    }
    if (sizeof(T) == 4)  // float-float partials of the FP32 kernel
        k_dsm_e_ff<<<cdiv(ctx->nym, 8), 256, 0, ctx->st>>>((const float4 *)ctx->dsm_part, nchunk, ctx->nyg,
                                                            ctx->avg_nu_t, dir, nchunk);
    else
        k_dsm_e<<<cdiv(ctx->nym, 8), 256, 0, ctx->st>>>(ctx->dsm_part, nchunk, ctx->nyg, ctx->avg_nu_t, dir, nchunk);
    count_launch(ctx, "k_dsm_e");
    // stage F (nu_t = max(-C(j)|S|/2, 0) everywhere) is left to the readers,
    // as after the one-pass kernel: |S| sits in the same canonical slot, the
    // fused RHS forms nu_t in its loader and the other readers (eqwm,
    // statistics, downloads) materialise it first
    ctx->nut_lazy = true;
    CF_CUDA(cudaGetLastError());
    return 0;
}

template int launch_dsm<double>(cf_ctx *, int);
template int launch_dsm<float>(cf_ctx *, int);
template int launch_nut_zero<double>(cf_ctx *);
template int launch_nut_materialize<double>(cf_ctx *);
template int launch_nut_materialize<float>(cf_ctx *);
template int launch_nut_wall_rows<double>(cf_ctx *);
template int launch_nut_wall_rows<float>(cf_ctx *);
template int launch_nut_zero<float>(cf_ctx *);

// z chunks of the multi-pass filter kernel: the count that minimises (waves
// of resident blocks) x (planes per chunk + the 2 halo planes a chunk loads
// again); its plane partials take ceil(nxp / 32) x nkc slots per row
int dsm_b_plan(int esz, int nxp, int nym, int nzp, int sms) {
    int per = 1;
    if (esz == 4)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dsm_b<float, true>, DB_X * DB_Y, dsm_b_smem<float, true>());
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dsm_b<double, false>, DB_X * DB_Y,
                                                      dsm_b_smem<double, false>());
    const long tiles = (long)cdiv(nxp, DB_X) * cdiv(nym, DB_Y), res = (long)(per < 1 ? 1 : per) * sms;
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
    return (int)best;
}

// shared-memory opt-in of the multi-pass filter kernel (two planes in dynamic
// shared memory; called at context creation)
int dsm_b_setup() {
    cudaFuncSetAttribute(k_dsm_b<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)dsm_b_smem<float, true>());
    cudaFuncSetAttribute(k_dsm_b<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)dsm_b_smem<float, false>());
    cudaFuncSetAttribute(k_dsm_b<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)dsm_b_smem<double, false>());
    return 0;
}
